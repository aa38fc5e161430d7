"""Device GMRES against the CPU oracle and the true FP64 residual."""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_C1, CFG_L3_K10, full_cfg

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_gmres_tolerance_c1(ls, ora):
    cfg = full_cfg(CFG_C1)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
    b = op.rhs()
    assert _rel(b, ref.rhs()) == 0.0
    x, hist, it, relres, code = op.gmres(b, max_iter=200, tol=1e-10)
    assert code == ls.LS_OK
    # The library's true residual and the oracle's agree, and meet the tolerance.
    r = b - ref.matvec(x)
    rr = np.linalg.norm(r) / np.linalg.norm(b)
    assert rr <= 2e-10
    assert abs(rr - relres) <= 1e-11
    xo, histo, ito, = ref.gmres(b, 200, 1e-10)
    assert abs(it - ito) <= 1
    assert _rel(x, xo) <= 1e-8
    # Residual estimates decrease monotonically (GMRES minimises the residual).
    assert np.all(np.diff(hist) <= 1e-14)
    op.close()


def test_gmres_restarted_matches_oracle(ls, ora):
    cfg = full_cfg(CFG_L3_K10)
    op = ls.Operator(cfg, device=0)
    ref = ora.Oracle(cfg.as_dict())
    b = op.rhs()
    for m, restarts in [(5, 1), (5, 2), (10, 1)]:
        x = op.gmres_restarted(b, m, restarts)
        xo = ref.gmres_restarted(b, m, restarts)
        assert _rel(x, xo) <= 1e-8


def test_gmres_not_converged_status(ls):
    op = ls.Operator(full_cfg(CFG_BUMPS), device=0)
    b = op.rhs()
    x, hist, it, relres, code = op.gmres(b, max_iter=2, tol=1e-14)
    assert code == ls.LS_E_NOT_CONVERGED
    assert it == 2 and np.isfinite(x).all()
    op.close()


def test_gmres_zero_rhs(ls):
    op = ls.Operator(full_cfg(CFG_L3_K10), device=0)
    x, hist, it, relres, code = op.gmres(np.zeros(op.N, dtype=np.complex128), max_iter=10, tol=1e-10)
    assert code == ls.LS_OK and np.all(x == 0)
    op.close()
