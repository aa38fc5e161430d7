"""GPU DAFMM matvec through the C ABI against the CPU oracle.

Bar: relative L2 difference <= 1e-10 against the oracle's restatement of
the reference DAFMM (same seeded inputs, same skeletons).
"""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_HFR, CFG_L3_K10, CFG_L5_BUMPS, full_cfg

pytestmark = pytest.mark.gpu

TOL_PARITY = 1e-10


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
        (CFG_C1, {"reference_rounding": 0}),
        (CFG_C1, {"yes2DFMM": 0}),
        (CFG_HFR, {}),
        (CFG_BUMPS, {}),
        (CFG_L3_K10, {"Qchoice": 2}),
        (CFG_L3_K10, {"Qchoice": 5, "nChebNodes": 5, "degreeOfBases": 5}),
        (CFG_L3_K10, {"nChebNodes": 8}),  # rank 64: the largest leaf, near-field GEMMs loop over 576 outputs
    ],
)
def test_matvec_matches_oracle(ls, ora, base, over):
    cfg = full_cfg(base, **over)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
    assert op.N == ref.N
    assert np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    x = _x(op.N, 11)
    y = op.matvec(x)
    yo = ref.matvec(x)
    assert _rel(y, yo) <= TOL_PARITY
    op.close()


def test_matvec_device_pointers_and_determinism(ls, ora):
    torch = pytest.importorskip("torch")
    cfg = full_cfg(CFG_C1)
    op = ls.Operator(cfg, device=0)
    x = _x(op.N, 3)
    xt = torch.from_numpy(x).to("cuda:0")
    y1 = torch.empty_like(xt)
    y2 = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), y1.data_ptr(), 0)
    op.matvec_device(xt.data_ptr(), y2.data_ptr(), 0)
    torch.cuda.synchronize()
    # Same inputs give bitwise identical outputs (no atomics in the matvec).
    assert torch.equal(y1, y2)
    yh = op.matvec(x)
    assert np.array_equal(y1.cpu().numpy(), yh)
    op.close()


def test_linearity_and_zero(ls):
    cfg = full_cfg(CFG_C1)
    op = ls.Operator(cfg, device=0)
    x1, x2 = _x(op.N, 1), _x(op.N, 2)
    a, b = 0.7 - 0.2j, -1.3 + 0.5j
    lhs = op.matvec(a * x1 + b * x2)
    rhs = a * op.matvec(x1) + b * op.matvec(x2)
    assert _rel(lhs, rhs) <= 1e-13
    assert np.all(op.matvec(np.zeros(op.N, dtype=np.complex128)) == 0)
    op.close()


def test_dense_oracle_small(ls, ora):
    """DAFMM vs the dense getMatrixEntry2 operator at small N. The GPU result
    must sit as close to the dense operator as the oracle's own DAFMM does;
    for a contrast that is nonzero on the whole domain the DAFMM error is at
    the NCA level."""
    for base, over, bound in [(CFG_L3_K10, {}, 1e-5), (CFG_L3_K10, {"Qchoice": 3, "TOL_POW": 10}, 1e-6)]:
        cfg = full_cfg(base, **over)
        op = ls.Operator(cfg, device=0)
        ref = ora.Oracle(cfg.as_dict())
        x = _x(op.N, 5)
        yd = ref.dense_matvec(x)
        e_gpu = _rel(op.matvec(x), yd)
        e_ora = _rel(ref.matvec(x), yd)
        assert e_gpu <= bound
        assert abs(e_gpu - e_ora) <= 1e-9
        op.close()


def test_empty_and_invalid(ls):
    with pytest.raises(ls.LSError) as ei:
        ls.Operator(ls.Config(nLevelsUniform=1), device=0)
    assert ei.value.code == ls.LS_E_INVALID
    with pytest.raises(ls.LSError):
        ls.Operator(ls.Config(Qchoice=6, bumps=()), device=0)
    op = ls.Operator(full_cfg(CFG_L3_K10), device=0)
    with pytest.raises(ValueError):
        op.matvec(np.zeros(3, dtype=np.complex128))
    op.close()


@pytest.mark.parametrize("name", ["l3_k10_gauss", "l4_k10_gauss", "l4_k24_flatbump"])
def test_matvec_matches_golden_fixtures(ls, name):
    import os
    import platform

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", platform.machine(), name + ".npz"))
    d = eval(str(g["cfg"]))  # dict literal written by tests/golden/make_golden.py
    op = ls.Operator(ls.Config(**{k: v for k, v in d.items()}), device=0)
    assert np.array_equal(op.skeleton_dump(), g["skeleton"])
    assert _rel(op.matvec(g["x"]), g["y"]) <= TOL_PARITY
    op.close()


def test_two_hfr_levels_match_oracle(ls, ora):
    """Level 5, kappa 40, three seeded bumps, NCA tolerance 1e-10 (the
    benchmark operator one level down): HFR at levels 3 and 2, so the
    cone-to-cone M2M (HFR_M2M_ILActiveTrue, G_FMM2DTree.hpp:3624-3710) and
    the HFR-to-HFR L2L (HFR_L2L_ILActiveTrue, :4021-4121), both folded
    through Atilde^-1 on the host, run on the GPU. Native FP64 and
    double-float kernels against the oracle's per-box QR solves, plus the
    FP32 operator's error bound."""
    torch = pytest.importorskip("torch")
    cfg = full_cfg(CFG_L5_BUMPS)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
    assert op.info["n_levels"] == 5 and op.info["level_LFR"] == 4
    assert np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    for seed in (11, 12):
        x = _x(op.N, seed)
        yo = ref.matvec(x)
        assert _rel(op.matvec(x), yo) <= TOL_PARITY
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
        assert _rel(op.matvec(x), yo) <= TOL_PARITY
        op.set_f64_kernels(ls.LS_F64_NATIVE)
    op.enable_f32()
    x = _x(op.N, 13)
    xt = torch.from_numpy(x).cuda()
    y32 = torch.empty_like(xt)
    op.matvec_device(xt.data_ptr(), y32.data_ptr(), 0, precision=ls.LS_PREC_F32)
    torch.cuda.synchronize()
    assert 1e-12 < _rel(y32.cpu().numpy(), ref.matvec(x)) <= 5e-5
    op.close()
