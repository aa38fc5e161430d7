"""The oracle's restated special functions and linear algebra against
independent implementations (numpy / scipy). CPU only."""
import numpy as np
import pytest


def test_gauss_legendre_order10(ora):
    nodes, w = ora.gauss_legendre(10)
    ref_x, ref_w = np.polynomial.legendre.leggauss(10)
    # The reference's table interleaves (-t, +t) pairs from the centre out.
    order = np.argsort(nodes)
    # numpy's double-precision rule is itself accurate to a few ulps (8.5e-16
    # in the weights on aarch64, where the oracle's long double is 128-bit).
    assert np.max(np.abs(nodes[order] - ref_x)) <= 1e-15
    assert np.max(np.abs(w[order] - ref_w)) <= 1e-15
    assert np.all(nodes[0::2] < 0) and np.all(nodes[1::2] > 0)
    assert np.allclose(nodes[0::2], -nodes[1::2], rtol=0, atol=0)
    assert abs(w.sum() - 2.0) <= 1e-15


@pytest.mark.parametrize("n", [0, 1, 2, 5, 9, 15, -1, -4, -15])
def test_bessel_against_scipy(ora, n):
    sp = pytest.importorskip("scipy.special")
    for x in [0.03, 0.4, 1.0, 2.5, 7.3, 19.0, 44.4, 113.0]:
        j, y = ora.bessel_jy(n, x)
        jr, yr = sp.jv(n, x), sp.yv(n, x)
        assert abs(j - jr) <= 1e-13 * max(1.0, abs(jr)), (n, x)
        assert abs(y - yr) <= 1e-12 * max(1.0, abs(yr)), (n, x)


@pytest.mark.parametrize("m,n", [(7, 7), (12, 5), (31, 21)])
def test_colpiv_qr_solve(ora, m, n):
    rng = np.random.default_rng(m * 100 + n)
    A = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
    b = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    x = ora.colpiv_solve(A, b)
    xr = np.linalg.lstsq(A, b, rcond=None)[0]
    assert np.linalg.norm(x - xr) <= 1e-12 * np.linalg.norm(xr)


def test_colpiv_rank_deficient_basic_solution(ora):
    # A rank-2 4x4 system: the solution reproduces b in the range of A.
    rng = np.random.default_rng(3)
    U = rng.standard_normal((4, 2)) + 1j * rng.standard_normal((4, 2))
    V = rng.standard_normal((2, 4)) + 1j * rng.standard_normal((2, 4))
    A = U @ V
    b = A @ (rng.standard_normal(4) + 0j)
    x = ora.colpiv_solve(A, b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert np.count_nonzero(np.abs(x) > 0) <= 2  # free variables set to zero


def test_bessel_order_recurrences_against_scipy(ora):
    """The far-field Hankel series takes J_n, Y_n (n <= 15) from J_0, J_1,
    Y_0, Y_1 by recurrence (forward for Y, forward or Miller's backward for
    J). Over the arguments kappa r of the far field it stays within 5e-14
    (J) and 1e-13 (Y) of max_n |.| of libstdc++'s per-order values, and
    within 2e-12 of scipy, the level at which libstdc++'s own per-order
    values differ from scipy's for arguments near 250."""
    sp = pytest.importorskip("scipy.special")
    n = np.arange(16)
    for x in np.concatenate([np.linspace(0.3, 20, 150), np.geomspace(20, 250, 120)]):
        J, Y = ora.bessel_jy_orders(15, x)
        pj = np.array([ora.bessel_jy(k, x)[0] for k in n])
        py = np.array([ora.bessel_jy(k, x)[1] for k in n])
        assert np.max(np.abs(J - pj)) <= 5e-14 * np.max(np.abs(pj)), x
        assert np.max(np.abs(Y - py)) <= 1e-13 * np.max(np.abs(py)), x
        rj, ry = sp.jv(n, x), sp.yv(n, x)
        assert np.max(np.abs(J - rj)) <= 2e-12 * np.max(np.abs(rj)), x
        assert np.max(np.abs(Y - ry)) <= 2e-12 * np.max(np.abs(ry)), x
