"""FP32 operator (FP32 blocks, FP32 accumulation) and the FP64 iterative
refinement around it (mixed-precision configuration)."""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_L3_K10, CFG_L5_BUMPS, full_cfg

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("base,over", [(CFG_BUMPS, {}), (CFG_L3_K10, {"nChebNodes": 8})])
def test_f32_matvec_error_is_single_precision(ls, ora, base, over):
    torch = pytest.importorskip("torch")
    cfg = full_cfg(base, **over)
    op = ls.Operator(cfg, device=0)
    op.enable_f32()
    x = np.random.default_rng(4).uniform(-1, 1, op.N) + 1j * np.random.default_rng(5).uniform(-1, 1, op.N)
    xt = torch.from_numpy(x).cuda()
    y32 = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), y32.data_ptr(), 0, precision=ls.LS_PREC_F32)
    torch.cuda.synchronize()
    y64 = op.matvec(x)
    e = _rel(y32.cpu().numpy(), y64)
    # FP32 storage and accumulation of the folded blocks. Folding Atilde^-1
    # into the blocks leaves cancellation that FP32 amplifies: the product is
    # good to ~1e-5 relative, far above FP64 and enough for the inner solves
    # of the FP64 refinement.
    assert 1e-12 < e <= 5e-5
    op.close()


def test_mixed_refinement_reaches_fp64_residual(ls, ora):
    cfg = full_cfg(CFG_C1)
    op = ls.Operator(cfg, device=0)
    op.enable_f32()
    b = op.rhs()
    x, hist, nmv, relres, code = op.gmres_mixed(b, max_outer=10, inner_iter=100, tol=1e-10)
    assert code == ls.LS_OK
    ref = ora.Oracle(cfg.as_dict())
    rr = np.linalg.norm(b - ref.matvec(x)) / np.linalg.norm(b)
    assert rr <= 2e-10
    assert abs(rr - relres) <= 1e-11
    x64, _, it64, _, _ = op.gmres(b, 200, 1e-10)
    assert _rel(x, x64) <= 1e-8
    op.close()


@pytest.mark.parametrize("base", [CFG_C1, CFG_L5_BUMPS])
def test_mixed_inner_basis_fp64_and_fp32(ls, ora, base):
    """FP64 refinement around inner GMRES on the FP32 operator, with the inner
    Arnoldi basis, Gram-Schmidt and Givens in FP64 (the default) or in FP32.
    Both reach the FP64 true residual 1e-8, checked with the oracle's
    operator; both solutions lie within 1e-7 of the plain FP64 GMRES
    solution (the distance the bench reports as mixed_rel_err_vs_fp64)."""
    cfg = full_cfg(base)
    op = ls.Operator(cfg, device=0)
    op.enable_f32()
    ref = ora.Oracle(cfg.as_dict())
    b = op.rhs()
    x64, _, it64, rr64, code64 = op.gmres(b, 400, 1e-10)
    assert code64 == ls.LS_OK
    out = {}
    for basis in (ls.LS_INNER_BASIS_F64, ls.LS_INNER_BASIS_F32):
        op.set_inner_basis(basis)
        x, hist, nmv, relres, code = op.gmres_mixed(b, max_outer=10, inner_iter=200, tol=1e-8)
        assert code == ls.LS_OK, basis
        rr = np.linalg.norm(b - ref.matvec(x)) / np.linalg.norm(b)
        assert rr <= 1.5e-8, (basis, rr)
        assert abs(rr - relres) <= 1e-10
        assert _rel(x, x64) <= 1e-7, (basis, _rel(x, x64))
        out[basis] = (nmv, _rel(x, x64))
    print("inner basis FP64 / FP32: applies and distance from FP64 GMRES", out)
    op.close()
