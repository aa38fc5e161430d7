"""Scattered field from the solved density (GMRES/GMRES.cpp:581-597) and the
Lippmann-Schwinger identity check (hybridTrueValidation_gmres.cpp:227-232)."""
import numpy as np
import pytest

from conftest import CFG_L3_K10, full_cfg

pytestmark = pytest.mark.gpu


def test_scattered_field_and_identity(ls, ora):
    # Flat-bump contrast: nonzero on the whole domain, so the q-scaled and
    # the bare operator are both accurate to the NCA tolerance.
    cfg = full_cfg(CFG_L3_K10, Qchoice=3, TOL_POW=10)
    op = ls.Operator(cfg, device=0)
    b = op.rhs()
    phi, hist, it, relres, code = op.gmres(b, max_iter=300, tol=1e-12)
    assert code == ls.LS_OK
    u_scat, u_tot, err = ls.scattered_field(cfg, phi)
    # The bare operator on the GPU matches the oracle's bare operator.
    ref = ora.Oracle(dict(cfg.as_dict(), findPhi=0))
    assert np.linalg.norm(u_scat - ref.matvec(phi)) <= 1e-10 * np.linalg.norm(u_scat)
    # phi solves (I + k^2 q G) phi = -k^2 q u_inc, hence phi / k^2 = -q u_tot
    # up to the two operators' NCA approximations of G.
    scale = np.linalg.norm(phi) / cfg.kappa ** 2
    assert err <= 1e-5 * scale
    op.close()
