import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ora():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ls():
    import lippmann_schwinger_solver_gb300 as pkg

    pkg.build()
    return pkg


# Small configurations the oracle assembles in seconds. The 256-leaf case is
# the reference's CPU-runnable configuration (uniform level 4, kappa 10,
# Gaussian contrast 1.5 exp(-160 |x|^2), NCA tolerance 1e-8).
CFG_L3_K10 = dict(nLevelsUniform=3, kappa=10.0, TOL_POW=8, Qchoice=0)
CFG_C1 = dict(nLevelsUniform=4, kappa=10.0, TOL_POW=8, Qchoice=0)
CFG_HFR = dict(nLevelsUniform=4, kappa=24.0, TOL_POW=10, Qchoice=3)  # level_LFR 3, HFR cones at level 2
CFG_BUMPS = dict(nLevelsUniform=4, kappa=40.0, TOL_POW=10, Qchoice=6)
# Level 5 at kappa 40: level_LFR 4, so HFR runs at levels 3 (16 cones) and
# 2 (32 cones) and the cone-to-cone M2M and the HFR-to-HFR L2L are used.
CFG_L5_BUMPS = dict(nLevelsUniform=5, kappa=40.0, TOL_POW=10, Qchoice=6)


def full_cfg(d, **over):
    import lippmann_schwinger_solver_gb300 as pkg

    d = dict(d)
    d.update(over)
    if d.get("Qchoice") == 6 and "bumps" not in d:
        d["bumps"] = pkg.seeded_bumps(20261203)
    return pkg.Config(**d)
