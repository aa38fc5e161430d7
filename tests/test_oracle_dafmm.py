"""The oracle's DAFMM against its golden fixtures and against the dense
getMatrixEntry2 operator; its two GMRES restatements. CPU only."""
import os

import numpy as np
import pytest

import platform

# Golden vectors written by tests/golden/make_golden.py on this architecture.
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", platform.machine())
BASE = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, degreeOfBases=6, findPhi=1, reference_rounding=1, L=1.0)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", ["l3_k10_gauss", "l4_k10_gauss", "l4_k24_flatbump"])
def test_oracle_reproduces_golden(ora, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = eval(str(g["cfg"]))  # a dict literal written by make_golden.py
    o = ora.Oracle(cfg)
    assert np.array_equal(o.skeleton_dump(), g["skeleton"])
    assert _rel(o.matvec(g["x"]), g["y"]) <= 1e-12
    assert _rel(o.rhs(), g["b"]) <= 1e-14


def test_dafmm_vs_dense_flat_contrast(ora):
    # A contrast that is nonzero on the whole domain: the DAFMM error is at
    # the NCA level.
    o = ora.Oracle(dict(BASE, nLevelsUniform=3, kappa=10.0, TOL_POW=10, Qchoice=3))
    x = np.random.default_rng(0).uniform(-1, 1, o.N) + 0.5j
    assert _rel(o.matvec(x), o.dense_matvec(x)) <= 1e-6


def test_dafmm_vs_dense_gaussian_contrast_gap(ora):
    # The reference's Gaussian contrast makes most far-field NCA blocks rank
    # 0 (entries below the absolute pivot threshold), which drops their
    # sources from coarser-level interactions: a documented property of the
    # reference algorithm, kept by the restatement.
    o = ora.Oracle(dict(BASE, nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0))
    x = np.random.default_rng(0).uniform(-1, 1, o.N) + 1j * np.random.default_rng(1).uniform(-1, 1, o.N)
    e = _rel(o.matvec(x), o.dense_matvec(x))
    assert 1e-7 < e < 1e-4


def test_gmres_variants_converge(ora):
    o = ora.Oracle(dict(BASE, nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0))
    b = o.rhs()
    x, hist, it = o.gmres(b, 100, 1e-10)
    assert hist[-1] <= 1e-10 and it < 100
    assert _rel(o.matvec(x), b) <= 1e-9
    assert np.all(np.diff(hist) <= 1e-15)
    x2 = o.gmres_restarted(b, 10, 2)
    assert _rel(o.matvec(x2), b) <= 1e-9
    assert _rel(x2, x) <= 1e-8


def test_scattered_field_operator(ora):
    # findPhi = 0 is the bare integral operator G used for the scattered
    # field (GMRES/GMRES.cpp:581-595): linear, no identity, no q scaling.
    o = ora.Oracle(dict(BASE, nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0, findPhi=0))
    x = np.random.default_rng(2).uniform(-1, 1, o.N) + 0j
    y = o.matvec(x)
    assert _rel(o.matvec(2.5 * x), 2.5 * y) <= 1e-14
    assert _rel(o.dense_matvec(x), y) <= 1e-2
