"""Post-processing helpers without a GPU: the density at arbitrary points by
the reference's Chebyshev-Q+ interpolation
(GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:187-219)
and the reference's result-file text (GMRES/GMRES.cpp:391-397)."""
import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_L3_K10, full_cfg


def _poly(x, y):
    # total degree 5 < degreeOfBases = 6: inside the span of the leaf bases
    return (1 + 2j) * x ** 5 - 0.7 * x ** 2 * y ** 3 + (0.3 - 1j) * x * y + 0.25 * y ** 4 - 1.5j


@pytest.mark.parametrize("base", [CFG_L3_K10, CFG_BUMPS])
def test_interpolation_reproduces_the_basis_span(ls, base):
    op = ls.Operator(full_cfg(base, nLevelsUniform=3), device=-1)
    pts = op.points()
    phi = _poly(pts[:, 0], pts[:, 1])
    rng = np.random.default_rng(3)
    xy = rng.uniform(-1, 1, (500, 2))
    xy[0] = (1.0, 1.0)     # upper corner: the last leaf
    xy[1] = (-1.0, -1.0)
    psi = op.interpolate(xy, phi)
    assert np.max(np.abs(psi - _poly(xy[:, 0], xy[:, 1]))) < 1e-11
    op.close()


def test_interpolation_matches_the_oracle_restatement(ls):
    from oracle import fno_oracle as fo
    cfg = full_cfg(CFG_BUMPS, nLevelsUniform=3)
    op = ls.Operator(cfg, device=-1)
    rng = np.random.default_rng(4)
    phi = rng.standard_normal(op.N) + 1j * rng.standard_normal(op.N)
    G = 32
    ix, iy = np.divmod(np.arange(G * G), G)
    xy = np.stack([cfg.L * (-1 + (2 * ix + 1) / G), cfg.L * (-1 + (2 * iy + 1) / G)], axis=1)
    psi = op.interpolate(xy, phi)
    ref = fo.grid_sample(op.points(), phi, cfg.L, G)
    assert np.linalg.norm(psi - ref) / np.linalg.norm(ref) < 1e-12
    with pytest.raises(ls.LSError) as e:
        op.interpolate(np.array([[0.0, 1.5]]), phi)
    assert e.value.code == ls.LS_E_INVALID
    op.close()


def test_result_file_text(ls, tmp_path):
    v = np.array([0.1 - 2j, 1e-7 + 123456789j, -0.5 + 0j, 3.14159265358979 - 2.5e-12j])
    p = tmp_path / "Phi_1_10"
    ls.write_result(str(p), v)
    lines = p.read_text().splitlines()
    assert lines == ["(%s,%s)" % ("%.6g" % z.real, "%.6g" % z.imag) for z in v]
    assert lines[0] == "(0.1,-2)" and lines[1] == "(1e-07,1.23457e+08)"
    back = np.array([complex(*map(float, s.strip("()").split(","))) for s in lines])
    assert np.allclose(back, v, rtol=1e-5, atol=1e-12)
    with pytest.raises(ls.LSError):
        ls.write_result(str(tmp_path / "no" / "such" / "dir"), v)
