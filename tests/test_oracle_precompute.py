"""The oracle's precomputations (far moments M, colleague near blocks)
against direct scipy integration. CPU only.

M = C Q^+ and B = V (i r^2/4) Q^+ with Q (36 x 21) of full column rank, so
C = M Q and V (i r^2/4) = B Q recover the integrals, which are compared
entry by entry with scipy.integrate. The reference integrates with an
adaptive 10x10 Gauss-Legendre rule to an absolute 1e-7
(FarFieldInteraction.hpp:37, NearFieldInteraction1.hpp:199); the bound
below allows for that.
"""
import numpy as np
import pytest


def _cheb_Q(n1=6, degree=6):
    k = np.arange(n1)
    c = -np.cos((k + 0.5) / n1 * np.pi)
    pts = [(c[i % n1], c[i // n1]) for i in range(n1 * n1)]
    bases = [(a, d - a) for d in range(degree) for a in range(d + 1)]
    Q = np.array([[np.cos(a * np.arccos(x)) * np.cos(b * np.arccos(y)) for (a, b) in bases] for (x, y) in pts])
    return Q, bases, pts


@pytest.fixture(scope="module")
def small_oracle(ora):
    cfg = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=3, Qchoice=0,
               findPhi=1, reference_rounding=0, L=1.0, kappa=10.0)
    return ora.Oracle(cfg)


def test_far_moments_against_scipy(small_oracle):
    integrate = pytest.importorskip("scipy.integrate")
    sp = pytest.importorskip("scipy.special")
    o = small_oracle
    M = o.far_moments()            # (36, 31): M[i, n + 15]
    Q, bases, _ = _cheb_Q()
    C = M.T @ Q                    # (31, 21)
    r = 1.0 / 2 ** o.nlevels
    kappa = 10.0
    for (n, l) in [(0, 0), (1, 2), (-3, 5), (7, 11), (-15, 20)]:
        a, b = bases[l]

        def f(y, x, part):
            R = np.hypot(x, y)
            th = np.arctan2(y, x)
            v = sp.jv(n, kappa * r * R) * np.exp(-1j * n * th) * np.cos(a * np.arccos(x)) * np.cos(b * np.arccos(y))
            return v.real if part == 0 else v.imag

        re = integrate.dblquad(f, -1, 1, -1, 1, args=(0,), epsabs=1e-12)[0]
        im = integrate.dblquad(f, -1, 1, -1, 1, args=(1,), epsabs=1e-12)[0]
        ref = r * r * (re + 1j * im)
        assert abs(C[n + 15, l] - ref) <= 3e-7 * r * r + 1e-12, (n, l)


def test_near_block_entries_against_scipy(small_oracle):
    integrate = pytest.importorskip("scipy.integrate")
    sp = pytest.importorskip("scipy.special")
    o = small_oracle
    B = o.near_blocks()            # (9, 36, 36)
    Q, bases, pts = _cheb_Q()
    kappa = 10.0
    r = 1.0 / 2 ** o.nlevels
    offs = [(-2, -2), (0, -2), (2, -2), (2, 0), (2, 2), (0, 2), (-2, 2), (-2, 0), (0, 0)]
    for (q, i, l) in [(8, 0, 0), (8, 14, 3), (3, 5, 1), (0, 35, 9)]:
        V = B[q] @ Q               # (36, 21) = V (i r^2 / 4)
        a, b = bases[l]
        X = (pts[i][0] - offs[q][0], pts[i][1] - offs[q][1])

        def f(y, x, part):
            R = np.hypot(X[0] - x, X[1] - y)
            v = sp.hankel1(0, kappa * r * R) * np.cos(a * np.arccos(x)) * np.cos(b * np.arccos(y))
            return v.real if part == 0 else v.imag

        # Split at the (possibly interior) singular point so each piece has
        # its log singularity on a corner.
        xs = sorted({-1.0, 1.0, min(max(X[0], -1.0), 1.0)})
        ys = sorted({-1.0, 1.0, min(max(X[1], -1.0), 1.0)})
        tot = 0j
        for x0, x1 in zip(xs[:-1], xs[1:]):
            for y0, y1 in zip(ys[:-1], ys[1:]):
                re = integrate.dblquad(f, x0, x1, y0, y1, args=(0,), epsabs=1e-11)[0]
                im = integrate.dblquad(f, x0, x1, y0, y1, args=(1,), epsabs=1e-11)[0]
                tot += re + 1j * im
        ref = tot * 1j * r * r / 4.0
        assert abs(V[i, l] - ref) <= 5e-7 * r * r, (q, i, l)


def test_reference_rounding_is_six_significant_digits(ora):
    cfg = dict(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=3, Qchoice=0,
               findPhi=1, L=1.0, kappa=10.0)
    raw = ora.Oracle(dict(cfg, reference_rounding=0))
    rnd = ora.Oracle(dict(cfg, reference_rounding=1))
    for A, Ar in [(raw.far_moments(), rnd.far_moments()), (raw.near_blocks(), rnd.near_blocks())]:
        for part in (np.real, np.imag):
            a, b = part(A).ravel(), part(Ar).ravel()
            expect = np.array([float("%.6g" % v) for v in a])
            assert np.array_equal(b, expect)
