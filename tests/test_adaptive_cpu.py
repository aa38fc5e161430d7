"""Adaptive quadtrees in the product's host assembly (ls_config.tree_adaptive).

At the configuration of the reference's published run (GMRES/Readme.md:43:
nCones_LFR 16, 6x6 nodes, epsilonTree 1e-5, L = 0.5, kappa = 40, TOL 1e-8,
Gaussian contrast) the product builds the same tree (N = 5,328, 5 levels,
level_LFR 4) and the same NCA skeletons, integer for integer, as the
oracle's adaptive restatement, whose matvec and RestartedGMRES reproduce the
README's residuals (tests/test_oracle_readme_residuals.py). No GPU needed."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

README = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5, Qchoice=0,
              findPhi=1, reference_rounding=1, L=0.5, kappa=40.0, tree_adaptive=1, treeAdaptivity=5)
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_skeletons(ora, d, adaptivity):
    L = ora.lib()
    L.ora_adaptive_skeletons.restype = ctypes.c_long
    L.ora_adaptive_skeletons.argtypes = [ctypes.POINTER(ora.OraCfg), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                         ctypes.c_long]
    c = ora.make_cfg(d)
    n = L.ora_adaptive_skeletons(ctypes.byref(c), adaptivity, None, 0)
    buf = np.empty(n, dtype=np.int32)
    L.ora_adaptive_skeletons(ctypes.byref(c), adaptivity, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
    return buf


def test_adaptive_host_assembly_matches_oracle_skeletons(ls, ora):
    # through the reference-shaped mirror (inputsToDFMM / userkernel / DFMM)
    inputs = ls.inputsToDFMM(nCones_LFR=16, nChebNodes=6, L=0.5, yes2DFMM=1, TOL_POW=8, degreeOfBases=6,
                             treeAdaptivity=5, treeAdaptive=1)
    S = ls.DFMM(inputs, ls.userkernel(kappa=40.0, Qchoice=0), device=-1)
    S.FMMTreeInitialisation()
    op = S.K
    assert op.N == 5328 and op.info["n_levels"] == 5 and op.info["level_LFR"] == 4
    assert np.array_equal(op.skeleton_dump(), _oracle_skeletons(ora, README, 5))
    a = ora.AdaptiveOracle(README, treeAdaptivity=5)
    assert np.array_equal(op.points(), a.points())
    op.close()
    a.close()


def test_adaptive_operator_refuses_uniform_only_entry_points(ls):
    op = ls.Operator(ls.Config(**README), device=-1)
    rc = ls.lib().ls_matvec_noalloc(op._h, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == ls.LS_E_STATE
    with pytest.raises(ls.LSError) as ei:
        op.interpolate(np.zeros((1, 2)), np.zeros(op.N, dtype=np.complex128))
    assert ei.value.code == ls.LS_E_STATE
    op.close()


# Further adaptive trees: the scattered-field operator (findPhi = 0) at
# kappa 20; a shallower tree (treeAdaptivity 4) at NCA tolerance 1e-10; 5 x 5
# nodes per leaf. Skeletons equal the oracle's in all of them; the TOL 1e-10
# tree sits at ~1e-11 from the oracle (measured 1.2e-11 and 1.6e-11), the
# rounding of the folded Atilde^-1 blocks against the oracle's per-box solves.
OTHER = [(dict(README, kappa=20.0, findPhi=0), 1e-12),
         (dict(README, kappa=20.0, TOL_POW=10, treeAdaptivity=4), 1e-10),
         (dict(README, nChebNodes=5, degreeOfBases=5), 1e-10)]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("cfg,bound", [(README, 1e-12)] + OTHER)
def test_adaptive_packed_program_in_bounds_and_equal_to_oracle(ls, ora, tmp_path, cfg, bound):
    """The packed gather-GEMV program of the adaptive operator -- every tile,
    gather index and output row the device kernels touch -- run on the host
    by tests/cpp/packed_program_check.cpp: all accesses in bounds, no output
    row written twice in a phase, no in-place phase reading a row it writes,
    and the result equal to the oracle's adaptive matvec."""
    exe = str(tmp_path / "packed_program_check")
    src = os.path.join(ROOT, "tests", "cpp", "packed_program_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                    src, "-o", exe], check=True, capture_output=True, timeout=600)
    cfg_path, x_path, y_path = (str(tmp_path / n) for n in ("cfg.bin", "x.bin", "y.bin"))
    with open(cfg_path, "wb") as f:
        f.write(bytes(ls.Config(**cfg).to_c()))
    a = ora.AdaptiveOracle(cfg, treeAdaptivity=cfg["treeAdaptivity"])
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, a.N) + 1j * rng.uniform(-1, 1, a.N)
    x.astype(np.complex128).tofile(x_path)
    out = subprocess.run([exe, cfg_path, x_path, y_path], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    y = np.fromfile(y_path, dtype=np.complex128)
    ya = a.matvec(x)
    a.close()
    assert np.linalg.norm(y - ya) / np.linalg.norm(ya) <= bound


@pytest.mark.parametrize("over,message", [
    (dict(treeAdaptivity=0), "treeAdaptivity"),
    (dict(treeAdaptivity=13), "treeAdaptivity"),
    (dict(nChebNodes=9), "nChebNodes"),
    (dict(degreeOfBases=12, nChebNodes=4), "degreeOfBases"),
    (dict(L=0.0), "L must be"),
    (dict(kappa=-1.0), "kappa"),
    (dict(TOL_POW=17), "TOL_POW"),
    (dict(Qchoice=7), "Qchoice"),
    # q resolved at once and kappa 0: a tree of fewer than 3 levels
    (dict(Qchoice=3, kappa=0.0, treeAdaptivity=1), "levels"),
])
def test_adaptive_config_rejections(ls, over, message):
    """Invalid adaptive configurations fail with LS_E_INVALID and a message
    naming the field, before any tree is built."""
    with pytest.raises(ls.LSError) as ei:
        ls.Operator(ls.Config(**dict(README, **over)), device=-1)
    assert ei.value.code == ls.LS_E_INVALID
    assert message in str(ei.value)
