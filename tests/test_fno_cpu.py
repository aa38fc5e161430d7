"""Learned preconditioner without a GPU: the network oracle's gradients
against finite differences, the library's host-side grid resampling weights
against the oracle's restatement of the reference's Chebyshev-Q+
interpolation, the grid contrast, the parameter layout, and the exported
symbols of include/ls_fno.h. No compute call runs on a device."""
import os
import re

import numpy as np
import pytest

from conftest import CFG_BUMPS, CFG_L3_K10, full_cfg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _declared():
    text = open(os.path.join(ROOT, "include", "ls_fno.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ls_\w+)\s*\(", text)))


def test_library_exports_every_fno_symbol(ls):
    L = ls.lib()
    names = _declared()
    assert set(names) == set(ls.FNO_SYMBOLS)
    for n in names:
        assert hasattr(L, n), n


def test_layout_matches_oracle(ls):
    from oracle import fno_oracle as fo
    for shape in [(128, 24, 4, 128), (32, 6, 2, 64)]:
        a = ls.fno_layout(*shape)
        b = fo.layout(*shape)
        assert a == b
    assert ls.fno_layout()["total"] == 9446114


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the error path without a GPU")
def test_create_without_gpu_fails_cleanly(ls):
    with pytest.raises(ls.LSError) as e:
        ls.FNO(grid=32, modes=6, layers=2, proj_width=64)
    assert e.value.code == ls.LS_E_CUDA


def test_oracle_gradient_matches_finite_differences():
    from oracle import fno_oracle as fo
    G, M, L, PW = 16, 4, 2, 32
    n = fo.layout(G, M, L, PW)["total"]
    rng = np.random.default_rng(5)
    p = rng.uniform(-0.3, 0.3, n)
    x = rng.uniform(-1, 1, (2, G * G, 6))
    t = rng.uniform(-1, 1, (2, G * G, 2))
    loss, g = fo.loss_and_grad(p, x, t, G, M, L, PW)
    assert np.isfinite(loss) and g.shape == (n,)
    for k in range(4):
        d = rng.standard_normal(n)
        eps = 1e-6
        lp, _ = fo.loss_and_grad(p + eps * d, x, t, G, M, L, PW)
        lm, _ = fo.loss_and_grad(p - eps * d, x, t, G, M, L, PW)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g @ d)


def test_oracle_bicubic_reproduces_quadratics():
    from oracle import fno_oracle as fo
    G, L = 32, 1.0
    ix, iy = np.divmod(np.arange(G * G), G)
    gx = L * (-1 + (2 * ix + 1) / G)
    gy = L * (-1 + (2 * iy + 1) / G)
    f = (1 + 2j) * gx ** 2 - 0.5 * gx * gy + (0.3 - 1j) * gy + 0.7
    rng = np.random.default_rng(1)
    pts = rng.uniform(-0.85, 0.85, (200, 2))
    want = (1 + 2j) * pts[:, 0] ** 2 - 0.5 * pts[:, 0] * pts[:, 1] + (0.3 - 1j) * pts[:, 1] + 0.7
    got = fo.grid_to_nodes(pts, f, L, G)
    assert np.max(np.abs(got - want)) < 1e-12


@pytest.mark.parametrize("base,grid", [(CFG_L3_K10, 32), (CFG_BUMPS, 64)])
def test_grid_weights_match_reference_interpolation(ls, base, grid):
    """psi(g) = sum_r w[g][r] phi[leaf(g)][r] from the library's host weights
    equals the oracle's leaf search + Q+ coefficients + Chebyshev sums."""
    from oracle import fno_oracle as fo
    cfg = full_cfg(base, nLevelsUniform=3)
    op = ls.Operator(cfg, device=-1)
    w, leaf = op.grid_weights(grid)
    rank = op.info["rank"]
    assert w.shape == (grid * grid, rank) and leaf.min() >= 0 and leaf.max() < op.info["n_leaves"]
    rng = np.random.default_rng(2)
    pts = op.points()
    # a smooth field, and an arbitrary one (checks the map, not the approximation)
    phi_s = np.exp(1j * cfg.kappa * 0.3 * pts[:, 0]) * (1 + pts[:, 1] ** 2)
    phi_r = rng.standard_normal(op.N) + 1j * rng.standard_normal(op.N)
    for phi in (phi_s, phi_r):
        psi = np.einsum("gr,gr->g", w.astype(np.float64), phi.reshape(-1, rank)[leaf])
        ref = fo.grid_sample(pts, phi, cfg.L, grid)
        assert np.linalg.norm(psi - ref) / np.linalg.norm(ref) < 2e-6
    # the smooth field is reproduced to interpolation accuracy
    ix, iy = np.divmod(np.arange(grid * grid), grid)
    gx = cfg.L * (-1 + (2 * ix + 1) / grid)
    gy = cfg.L * (-1 + (2 * iy + 1) / grid)
    exact = np.exp(1j * cfg.kappa * 0.3 * gx) * (1 + gy ** 2)
    psi = np.einsum("gr,gr->g", w.astype(np.float64), phi_s.reshape(-1, rank)[leaf])
    assert np.linalg.norm(psi - exact) / np.linalg.norm(exact) < 1e-3
    op.close()


def test_grid_contrast_is_the_plugin(ls):
    cfg = full_cfg(CFG_BUMPS, nLevelsUniform=3)
    op = ls.Operator(cfg, device=-1)
    G = 16
    q = op.grid_contrast(G)
    ix, iy = np.divmod(np.arange(G * G), G)
    gx = -1 + (2 * ix + 1) / G
    gy = -1 + (2 * iy + 1) / G
    want = sum(a * np.exp(-((gx - cx) ** 2 + (gy - cy) ** 2) / w ** 2) for cx, cy, a, w in cfg.bumps)
    assert np.allclose(q, want, rtol=1e-6, atol=1e-7)
    with pytest.raises(ls.LSError):
        op.grid_contrast(12)
    op.close()


def test_host_only_operator_refuses_device_grid_calls(ls):
    op = ls.Operator(full_cfg(CFG_L3_K10), device=-1)
    with pytest.raises(ls.LSError) as e:
        op.grid_sample_device(32, 1, 0, 0)
    assert e.value.code in (ls.LS_E_INVALID, ls.LS_E_STATE)
    b = np.ones(op.N, dtype=complex)
    with pytest.raises(ls.LSError) as e:
        op.fgmres_nn(None, b, flags=0)
    assert e.value.code == ls.LS_E_STATE
    op.close()


def test_many_scatterer_specs_are_seeded_and_in_range():
    from lippmann_schwinger_solver_gb300 import scatterers as sc
    a = sc.scatterer_specs(32, 20261203)
    assert a == sc.scatterer_specs(32, 20261203)
    assert {lv for lv, _, _ in a} == {4, 5, 6}
    for lv, k, bumps in a:
        assert 10.0 <= k <= 60.0 and 1 <= len(bumps) <= 4
        for cx, cy, amp, w in bumps:
            assert -0.6 <= cx <= 0.6 and -0.6 <= cy <= 0.6 and 0.5 <= amp <= 1.5 and 0.05 <= w <= 0.2
    cfg = sc.config(*a[0])
    assert cfg.Qchoice == 6 and cfg.nLevelsUniform == a[0][0] and cfg.kappa == a[0][1]


def test_training_data_generators(ls):
    from lippmann_schwinger_solver_gb300 import fno_train as ft
    rng = np.random.default_rng(3)
    for _ in range(20):
        kappa, bumps = ft.scatterer(rng)
        assert 10.0 <= kappa <= 40.0 and 1 <= len(bumps) <= 4
    op = ls.Operator(ft.operator_config(20.0, [(0.1, 0.2, 1.0, 0.1)], 3, 8), device=-1)
    B = ft.off_shell_rhs(op, 20.0, 5, np.random.default_rng(4))
    assert B.shape == (op.N, 5) and B.flags["F_CONTIGUOUS"]
    q = op.contrast()
    # each column is -kappa^2 q times a unit-modulus wave
    assert np.allclose(np.abs(B), (20.0 ** 2) * np.abs(q)[:, None], rtol=1e-12, atol=1e-300)
    op.close()
