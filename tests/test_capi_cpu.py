"""The C ABI library without a GPU: it loads, exports every symbol declared
in include/ls_dafmm.h, and its host assembly (device < 0) reproduces the
oracle's precomputations and NCA skeletons exactly. No compute call runs."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_HFR, CFG_L3_K10, full_cfg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "ls_dafmm.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ls_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(ls):
    L = ls.lib()
    names = _declared()
    assert len(names) >= 18
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(ls.EXPORTED_SYMBOLS)
    assert b"sm_103a" in L.ls_version()


@pytest.mark.parametrize("cap", ["0", "150"])
def test_hankel_table_overflow_matches_oracle(ls, ora, monkeypatch, cap):
    """The assembler shares far-field Hankel vectors through a table of
    bounded size; past the bound (here forced to 0 and 150 vectors) tasks
    compute and keep their own. Skeletons stay identical to the oracle's,
    which computes every vector itself."""
    monkeypatch.setenv("LS_HANKEL_TABLE_CAP", cap)
    cfg = full_cfg(CFG_HFR)
    op = ls.Operator(cfg, device=-1)
    assert np.array_equal(op.skeleton_dump(), ora.Oracle(cfg.as_dict()).skeleton_dump())
    op.close()


@pytest.mark.parametrize("base,over", [
    (CFG_L3_K10, {}),
    (CFG_C1, {}),
    (CFG_C1, {"findPhi": 0}),
    (CFG_C1, {"yes2DFMM": 0}),
    (CFG_HFR, {}),
    (CFG_BUMPS, {"nLevelsUniform": 3}),
    (CFG_L3_K10, {"Qchoice": 4, "TOL_POW": 6}),
    (CFG_L3_K10, {"Qchoice": 1}),
])
def test_host_assembly_matches_oracle(ls, ora, base, over):
    cfg = full_cfg(base, **over)
    op = ls.Operator(cfg, device=-1)
    ref = ora.Oracle(cfg.as_dict())
    assert op.N == ref.N
    assert op.info["level_LFR"] == ref.level_lfr
    assert np.array_equal(op.skeleton_dump(), ref.skeleton_dump())
    M, B = op.precomputations()
    assert np.array_equal(M, ref.far_moments())
    assert np.array_equal(B, ref.near_blocks())
    assert np.array_equal(op.points(), ref.points())
    assert np.array_equal(op.contrast(), ref.contrast())
    assert np.array_equal(op.rhs(), ref.rhs())
    op.close()


def test_host_only_operator_refuses_device_calls(ls):
    op = ls.Operator(full_cfg(CFG_L3_K10), device=-1)
    x = np.zeros(op.N, dtype=np.complex128)
    with pytest.raises(ls.LSError) as ei:
        op.matvec(x)
    assert ei.value.code == ls.LS_E_STATE
    with pytest.raises(ls.LSError) as ei:
        op.gmres(x, 5, 1e-3)
    assert ei.value.code == ls.LS_E_STATE
    with pytest.raises(ls.LSError) as ei:
        op.enable_f32()
    assert ei.value.code == ls.LS_E_STATE
    with pytest.raises(ls.LSError) as ei:
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
    assert ei.value.code == ls.LS_E_STATE
    with pytest.raises(ls.LSError) as ei:  # an unknown kernel choice is rejected first
        op.set_f64_kernels(5)
    assert ei.value.code == ls.LS_E_INVALID
    with pytest.raises(ls.LSError) as ei:
        op.gmres_mixed_batched(np.zeros((op.N, 3), dtype=np.complex128))
    assert ei.value.code == ls.LS_E_STATE
    assert op.tc_stages() == 0  # no tensor-core form without a device
    info = op.info
    assert info["far_entries"] > 0 and info["matvec_flops"] > 8 * info["far_entries"]
    assert info["m2l_entries"] <= info["far_entries"]
    # Stage times: six non-negative laps that add up to the total.
    stages = info["assemble_stage_seconds"]
    assert len(stages) == 6 and min(stages) >= 0.0 and stages[3] > 0.0
    assert sum(stages) == pytest.approx(info["assemble_seconds"], rel=1e-3, abs=1e-3)
    op.close()


@pytest.mark.parametrize("over,msg", [
    ({"nLevelsUniform": 1}, "nLevelsUniform"),
    ({"nLevelsUniform": 2}, "nLevelsUniform"),
    ({"nLevelsUniform": 11}, "nLevelsUniform"),
    ({"nChebNodes": 1}, "nChebNodes"),
    ({"degreeOfBases": 9}, "degreeOfBases"),
    ({"Qchoice": 7}, "Qchoice"),
    ({"L": 0.0}, "L must"),
    ({"TOL_POW": 0}, "TOL_POW"),
])
def test_invalid_configurations_are_rejected(ls, over, msg):
    with pytest.raises(ls.LSError) as ei:
        ls.Operator(full_cfg(CFG_L3_K10, **over), device=-1)
    assert ei.value.code == ls.LS_E_INVALID
    assert msg in str(ei.value)


def test_bumps_contrast_needs_bumps(ls):
    with pytest.raises(ls.LSError) as ei:
        ls.Operator(ls.Config(Qchoice=6, nLevelsUniform=3), device=-1)
    assert ei.value.code == ls.LS_E_INVALID


def test_seeded_bumps_are_reproducible(ls):
    a = ls.seeded_bumps(20261203)
    assert a == ls.seeded_bumps(20261203)
    for cx, cy, amp, w in a:
        assert -0.6 <= cx <= 0.6 and -0.6 <= cy <= 0.6 and 0.5 <= amp <= 1.5 and 0.05 <= w <= 0.2


def test_null_handles_do_not_crash(ls):
    L = ls.lib()
    assert L.ls_op_destroy(None) == 0
    assert L.ls_op_info(None, None) == ls.LS_E_INVALID
    assert L.ls_matvec(None, None, None, None) == ls.LS_E_INVALID
    assert L.ls_op_skeleton_dump(None, None, 0) == -1
    assert L.ls_op_tc_stages(None, None) == ls.LS_E_INVALID
    assert L.ls_tc_wait_probe(0, 1000, None) == ls.LS_E_INVALID
    v = ctypes.c_int()
    assert L.ls_tc_wait_probe(0, 0, ctypes.byref(v)) == ls.LS_E_INVALID


@pytest.mark.parametrize("n", [0, 8, 24, 272])
def test_mma_issue_measure_rejects_shapes_before_any_device_call(ls, n):
    """N must be a multiple of 16 in [16, 256]; the check comes before the
    device lookup, so it answers without a GPU."""
    with pytest.raises(ls.LSError) as ei:
        ls.measure_mma_issue(0, n)
    assert ei.value.code == ls.LS_E_INVALID


def test_noalloc_rejects_operators_larger_than_its_static_array(ls):
    """The allocation-free matvec checks the operator's scratch size first:
    a level-7 operator needs more than LS_STATIC_SCRATCH_ELEMS (2^20)
    complex entries and is rejected with LS_E_INVALID, also when it was
    assembled on the host only."""
    import ctypes

    op = ls.Operator(ls.Config(nLevelsUniform=7, kappa=10.0, TOL_POW=4, Qchoice=0), device=-1)
    rc = ls.lib().ls_matvec_noalloc(op._h, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == ls.LS_E_INVALID
    assert b"static array holds 1048576" in ls.lib().ls_last_error()
    small = ls.Operator(ls.Config(nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0), device=-1)
    assert ls.lib().ls_matvec_noalloc(small._h, ctypes.c_void_p(16), ctypes.c_void_p(16), None) == ls.LS_E_STATE
    op.close()
    small.close()


def test_rhs_angles_is_the_turned_reference_rhs(ls):
    """ls_op_rhs_angles: column t is -kappa^2 q exp(i kappa (x cos t + y sin t))
    (GMRES/GMRES.cpp:122-125 turned by t), the t = 0 column is ls_op_rhs bit
    for bit, and bad arguments are rejected."""
    op = ls.Operator(full_cfg(CFG_L3_K10), device=-1)
    th = np.array([0.0, 0.7, np.pi, 5.9])
    B = op.rhs_angles(th)
    assert B.shape == (op.N, 4) and B.flags["F_CONTIGUOUS"]
    assert np.array_equal(B[:, 0], op.rhs())
    xy, q, k = op.points(), op.contrast(), op.cfg.kappa
    ref = -(k * k) * q[:, None] * np.exp(1j * k * (np.outer(xy[:, 0], np.cos(th)) + np.outer(xy[:, 1], np.sin(th))))
    assert np.max(np.abs(B - ref)) <= 1e-14 * np.max(np.abs(ref))
    L = ls.lib()
    out = np.empty(2 * op.N)
    t0 = np.zeros(1)
    assert L.ls_op_rhs_angles(op._h, None, 1, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == ls.LS_E_INVALID
    assert L.ls_op_rhs_angles(op._h, t0.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 0,
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == ls.LS_E_INVALID
    op.close()
