"""Numeric pin of the oracle to the reference's own published output.

GMRES/Readme.md:43-101 publishes the run
  ./testFMM2D_GMRES 16 6 5 0.5 40.0 1 6 8 10 1 5 0
(nCones_LFR 16, 6x6 Chebyshev nodes, adaptive tree with epsilonTree 1e-5,
L = 0.5, kappa = 40, directional FMM, degree-6 bases, NCA tolerance 1e-8,
Gaussian contrast 1.5 exp(-160 |x|^2)) and, for RestartedGMRES with m = 10,
the relative residual |b - A x| / |b| printed with six significant digits:
  "GMRES Solver 1,10 ... Err in GMRES: 4.59412e-06"   (GMRES/Readme.md:64-65)
  "GMRES Solver 2,10 ... Err in GMRES: 1.28443e-10"   (GMRES/Readme.md:84-85)
The adaptive-tree restatement (oracle/ls_oracle_adaptive.cpp: tree, 2:1
level restriction, NCA, every matvec phase with leaves on several levels and
the four near-neighbour kinds, RestartedGMRES) reproduces both numbers to
the printed digits. The tolerance below (2e-5 relative) is two units of the
sixth printed digit; the (1, 50) residual is at the FP64 round-off floor
(1.4e-15 published), where summation order decides the digits, so it is only
bounded.

The second test closes the chain to the GPU product: on uniform trees the
same restatement equals the uniform oracle (oracle/ls_oracle.cpp, the one
the CUDA operator is checked against at <= 1e-10) to round-off.
"""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_HFR, full_cfg

README_CFG = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5, Qchoice=0,
                  findPhi=1, reference_rounding=1, L=0.5, kappa=40.0, n_bumps=0)


def test_readme_gmres_residuals_reproduced(ora):
    o = ora.AdaptiveOracle(README_CFG, treeAdaptivity=5)
    assert o.N == 5328 and o.unmatched_neighbors == 0
    b = o.rhs()
    for restarts, m, published in [(1, 10, 4.59412e-06), (2, 10, 1.28443e-10)]:
        x = o.gmres_restarted(b, m, restarts)
        res = np.linalg.norm(b - o.matvec(x)) / np.linalg.norm(b)
        assert abs(res / published - 1.0) <= 2e-5, (restarts, m, res, published)
    x = o.gmres_restarted(b, 50, 1)
    res = np.linalg.norm(b - o.matvec(x)) / np.linalg.norm(b)
    assert res <= 1e-14, res
    o.close()


@pytest.mark.parametrize("base,over", [(CFG_C1, {}), (CFG_HFR, {}), (CFG_BUMPS, {}), (CFG_C1, {"findPhi": 0})])
def test_adaptive_restatement_on_uniform_trees_equals_uniform_oracle(ora, base, over):
    d = full_cfg(base, **over).as_dict()
    a = ora.AdaptiveOracle(d, treeAdaptivity=-1)
    u = ora.Oracle(d)
    assert a.N == u.N
    x = np.random.default_rng(5).uniform(-1, 1, a.N) + 1j * np.random.default_rng(6).uniform(-1, 1, a.N)
    ya, yu = a.matvec(x), u.matvec(x)
    assert np.linalg.norm(ya - yu) / np.linalg.norm(yu) <= 1e-13
    a.close()
    u.close()
