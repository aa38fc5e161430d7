"""Double-float kernels behind the FP64 entry points (LS_F64_DOUBLE_FLOAT).

The operator is the same; its entries, charges and potentials are held as
FP32 hi/lo pairs (48-bit significand) and multiplied and summed with
error-free FP32 transformations. Bars, written per test:
  * against the oracle's DAFMM: the parity bar of the FP64 path, 1e-10;
  * against the native FP64 kernels on the same operator: 2e-11. The
    arithmetic carries about 2^-48 (3.6e-15) per entry and per accumulation
    step, against 2^-53 for FP64; cancellation between the near and far
    contributions amplifies both. Measured: 1e-14 (Lippmann-Schwinger
    operator, level 4, kappa 10) to 4e-12 (bare Helmholtz operator G,
    findPhi = 0, where nothing of the size of the identity is added).
"""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_HFR, CFG_L3_K10, full_cfg

pytestmark = pytest.mark.gpu

TOL_PARITY = 1e-10
TOL_VS_NATIVE = 2e-11


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _x(n, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)


@pytest.mark.parametrize(
    "base,over",
    [
        (CFG_L3_K10, {}),
        (CFG_C1, {}),
        (CFG_C1, {"findPhi": 0}),
        (CFG_HFR, {}),
        (CFG_BUMPS, {}),
        (CFG_L3_K10, {"nChebNodes": 8}),
    ],
)
def test_double_float_matches_oracle_and_native(ls, ora, base, over):
    cfg = full_cfg(base, **over)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
    x = _x(op.N, 21)
    y64 = op.matvec(x)
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    ydf = op.matvec(x)
    yo = ref.matvec(x)
    e_ora, e_nat = _rel(ydf, yo), _rel(ydf, y64)
    print(f"double-float vs oracle {e_ora:.2e}, vs native FP64 {e_nat:.2e}")
    assert e_ora <= TOL_PARITY
    assert e_nat <= TOL_VS_NATIVE
    # Switching back restores the native kernels bit for bit.
    op.set_f64_kernels(ls.LS_F64_NATIVE)
    assert np.array_equal(op.matvec(x), y64)
    op.close()


def test_double_float_device_pointers_deterministic(ls):
    torch = pytest.importorskip("torch")
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    x = _x(op.N, 5)
    xt = torch.from_numpy(x).to("cuda:0")
    y1 = torch.empty_like(xt)
    y2 = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), y1.data_ptr(), 0)
    op.matvec_device(xt.data_ptr(), y2.data_ptr(), 0)
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
    assert np.array_equal(y1.cpu().numpy(), op.matvec(x))
    # In place (x and y the same buffer) gives the same product.
    op.matvec_device(xt.data_ptr(), xt.data_ptr(), 0)
    torch.cuda.synchronize()
    assert torch.equal(xt, y1)
    op.close()


def test_double_float_gmres_reaches_fp64_residual(ls):
    op = ls.Operator(full_cfg(CFG_C1), device=0)
    b = op.rhs()
    x64, _, it64, rr64, code64 = op.gmres(b, max_iter=200, tol=1e-10)
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    xdf, _, itdf, rrdf, codedf = op.gmres(b, max_iter=200, tol=1e-10)
    assert code64 == 0 and codedf == 0
    assert abs(itdf - it64) <= 1
    # Judge with the native FP64 operator.
    op.set_f64_kernels(ls.LS_F64_NATIVE)
    r = b - op.matvec(xdf)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 2e-10
    assert _rel(xdf, x64) <= 1e-8
    op.close()


def test_set_f64_kernels_rejects_unknown(ls):
    op = ls.Operator(full_cfg(CFG_L3_K10), device=0)
    with pytest.raises(ls.LSError):
        op.set_f64_kernels(7)
    op.close()
