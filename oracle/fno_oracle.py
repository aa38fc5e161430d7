"""ORACLE - TEST INFRASTRUCTURE ONLY.

CPU restatement, in float64, of the learned preconditioner's arithmetic:
the spectral neural operator (forward, loss and - through autograd - its
gradients), the Adam update, the training-batch construction, and the
grid resampling between the Chebyshev nodes and the network's grid. Only
tests/ and __graft_entry__.smoke() use it, as the checker of the CUDA
kernels (csrc/fno.cu, csrc/nn_precond.cu).

The network is written here the textbook way - torch.fft.rfft2 / irfft2 of
the whole grid, keep the two corner blocks of modes, multiply, transform
back - which is an independent formulation of the truncated DFTs that the
CUDA kernels form directly. torch runs on the CPU only.

The nodes -> grid map restates the reference's Chebyshev-Q+ interpolation
(GMRES_Hybrid/LippmannSchwinger/main/hybridTrueValidation_gmres.cpp:187-219):
the leaf that contains a point is found by its bounds, c = Q+ phi_leaf with
Q the 36 x 21 matrix of T_a(x) T_b(y) at the leaf's Chebyshev nodes, and
psi = sum_l c_l T_a(l)(x') T_b(l)(y'). Q+ is taken here from numpy's pinv
(the reference uses Q_pinv2 from its own decomposition; both are the
Moore-Penrose inverse of a full-column-rank Q).
"""
import numpy as np
import torch

WIDTH = 32
IN_CH = 6
OUT_CH = 2


def layout(grid, modes, layers, proj):
    o, lay = 0, {}

    def take(name, n):
        nonlocal o
        lay[name] = (o, n)
        o += n
    take("lift_w", WIDTH * IN_CH)
    take("lift_b", WIDTH)
    for l in range(layers):
        take(f"spec{l}", 2 * (2 * modes) * modes * WIDTH * WIDTH)
        take(f"pw_w{l}", WIDTH * WIDTH)
        take(f"pw_b{l}", WIDTH)
    take("p1_w", proj * WIDTH)
    take("p1_b", proj)
    take("p2_w", OUT_CH * proj)
    take("p2_b", OUT_CH)
    lay["total"] = o
    return lay


def _unpack(p, grid, modes, layers, proj):
    lay = layout(grid, modes, layers, proj)

    def g(name, shape):
        o, n = lay[name]
        return p[o:o + n].reshape(shape)
    P = {"lift_w": g("lift_w", (WIDTH, IN_CH)), "lift_b": g("lift_b", (WIDTH,)),
         "p1_w": g("p1_w", (proj, WIDTH)), "p1_b": g("p1_b", (proj,)),
         "p2_w": g("p2_w", (OUT_CH, proj)), "p2_b": g("p2_b", (OUT_CH,))}
    for l in range(layers):
        s = g(f"spec{l}", (2 * modes, modes, WIDTH, WIDTH, 2))
        P[f"spec{l}"] = torch.complex(s[..., 0], s[..., 1])
        P[f"pw_w{l}"] = g(f"pw_w{l}", (WIDTH, WIDTH))
        P[f"pw_b{l}"] = g(f"pw_b{l}", (WIDTH,))
    return P


def _gelu(x):
    return 0.5 * x * (1.0 + torch.erf(x / np.sqrt(2.0)))


def _forward_t(p, x, grid, modes, layers, proj, ssq=None):
    """p: float64 tensor of parameters; x: [B, G*G, 6]; returns [B, G*G, 2]."""
    B, G, M = x.shape[0], grid, modes
    P = _unpack(p, grid, modes, layers, proj)
    xin = x.reshape(B, G, G, IN_CH)
    if ssq is not None:
        sc = 1.0 / torch.sqrt(ssq / (G * G))
        xin = xin.clone()
        xin[..., 1:3] = xin[..., 1:3] * sc[:, None, None, None]
    h = xin @ P["lift_w"].T + P["lift_b"]
    for l in range(layers):
        hc = h.permute(0, 3, 1, 2)
        X = torch.fft.rfft2(hc)
        W = P[f"spec{l}"]
        out_ft = torch.zeros(B, WIDTH, G, G // 2 + 1, dtype=X.dtype)
        out_ft[:, :, :M, :M] = torch.einsum("bixy,xyio->boxy", X[:, :, :M, :M], W[:M])
        out_ft[:, :, G - M:, :M] = torch.einsum("bixy,xyio->boxy", X[:, :, G - M:, :M], W[M:])
        s = torch.fft.irfft2(out_ft, s=(G, G)).permute(0, 2, 3, 1)
        z = s + h @ P[f"pw_w{l}"].T + P[f"pw_b{l}"]
        h = _gelu(z) if l + 1 < layers else z
    out = _gelu(h @ P["p1_w"].T + P["p1_b"]) @ P["p2_w"].T + P["p2_b"]
    if ssq is not None:
        out = out * torch.sqrt(ssq / (G * G))[:, None, None, None]
    return out.reshape(B, G * G, OUT_CH)


def forward(params, x, grid, modes, layers, proj, ssq=None):
    p = torch.tensor(np.asarray(params, dtype=np.float64))
    xt = torch.tensor(np.asarray(x, dtype=np.float64))
    st = None if ssq is None else torch.tensor(np.asarray(ssq, dtype=np.float64))
    with torch.no_grad():
        return _forward_t(p, xt, grid, modes, layers, proj, st).numpy()


def loss_and_grad(params, x, target, grid, modes, layers, proj):
    """mean_b |o_b - t_b|^2 / |t_b|^2 and its gradient (flat float64)."""
    p = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    xt = torch.tensor(np.asarray(x, dtype=np.float64))
    tt = torch.tensor(np.asarray(target, dtype=np.float64))
    o = _forward_t(p, xt, grid, modes, layers, proj)
    B = xt.shape[0]
    num = ((o - tt) ** 2).reshape(B, -1).sum(1)
    den = (tt ** 2).reshape(B, -1).sum(1)
    loss = (num / den).mean()
    loss.backward()
    return float(loss.detach()), p.grad.numpy().copy()


def adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (t = step number, from 1)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    return p, m, v


def make_batch(F, PHI, Q, kap, sidx, coef, grid):
    """Training batch: F, PHI [S, nb, G*G] complex; Q [S, G*G]; kap [S];
    sidx [B]; coef [B, nb] complex. Returns in [B, G*G, 6], target [B, G*G, 2]."""
    G = grid
    B = len(sidx)
    ix, iy = np.divmod(np.arange(G * G), G)
    xs = -1.0 + (2.0 * ix + 1.0) / G
    ys = -1.0 + (2.0 * iy + 1.0) / G
    inp = np.zeros((B, G * G, IN_CH))
    tgt = np.zeros((B, G * G, OUT_CH))
    for b in range(B):
        s = sidx[b]
        f = coef[b] @ F[s]
        t = coef[b] @ PHI[s]
        sc = 1.0 / np.sqrt(np.sum(np.abs(f) ** 2) / (G * G))
        inp[b, :, 0] = Q[s]
        inp[b, :, 1] = f.real * sc
        inp[b, :, 2] = f.imag * sc
        inp[b, :, 3] = kap[s]
        inp[b, :, 4] = xs
        inp[b, :, 5] = ys
        tgt[b, :, 0] = t.real * sc
        tgt[b, :, 1] = t.imag * sc
    return inp, tgt


def cheb_t(x, n):
    return np.cos(n * np.arccos(np.clip(x, -1.0, 1.0)))


def grid_sample(points, phi, L, grid, n_cheb=6, degree=6):
    """psi at the G x G grid points from the node values phi (leaf order,
    n_cheb^2 nodes per leaf, node = row * n + col), the reference's
    Chebyshev-Q+ interpolation."""
    rank = n_cheb * n_cheb
    nleaf = len(phi) // rank
    cheb = -np.cos((np.arange(n_cheb) + 0.5) / n_cheb * np.pi)
    bases = [(a, d - a) for d in range(degree) for a in range(d + 1)]
    Q = np.array([[cheb_t(cheb[i % n_cheb], a) * cheb_t(cheb[i // n_cheb], b) for (a, b) in bases]
                  for i in range(rank)])
    Qp = np.linalg.pinv(Q)
    pts = points.reshape(nleaf, rank, 2)
    lo = pts.min(axis=1)
    hi = pts.max(axis=1)
    centre = 0.5 * (lo + hi)
    side = int(round(np.sqrt(nleaf)))
    rad = L / side
    ix, iy = np.divmod(np.arange(grid * grid), grid)
    gx = L * (-1.0 + (2.0 * ix + 1.0) / grid)
    gy = L * (-1.0 + (2.0 * iy + 1.0) / grid)
    out = np.zeros(grid * grid, dtype=complex)
    coef = np.einsum("lr,tr->tl", Qp, phi.reshape(nleaf, rank))
    for g in range(grid * grid):
        inside = np.nonzero((centre[:, 0] - rad <= gx[g]) & (gx[g] < centre[:, 0] + rad) &
                            (centre[:, 1] - rad <= gy[g]) & (gy[g] < centre[:, 1] + rad))[0]
        t = inside[0]
        px = (gx[g] - centre[t, 0]) / rad
        py = (gy[g] - centre[t, 1]) / rad
        out[g] = sum(coef[t, l] * cheb_t(px, a) * cheb_t(py, b) for l, (a, b) in enumerate(bases))
    return out


def _catmull_rom(t):
    t2, t3 = t * t, t * t * t
    return np.stack([0.5 * (-t3 + 2 * t2 - t), 0.5 * (3 * t3 - 5 * t2 + 2),
                     0.5 * (-3 * t3 + 4 * t2 + t), 0.5 * (t3 - t2)], axis=-1)


def grid_to_nodes(points, f, L, grid):
    """Bicubic (Catmull-Rom, clamped at the border) interpolation of the grid
    field f [G*G] complex at the points [n, 2]."""
    G = grid
    F = f.reshape(G, G)
    u = (points[:, 0] / L + 1.0) * 0.5 * G - 0.5
    v = (points[:, 1] / L + 1.0) * 0.5 * G - 0.5
    u0, v0 = np.floor(u), np.floor(v)
    wu, wv = _catmull_rom(u - u0), _catmull_rom(v - v0)
    out = np.zeros(len(points), dtype=complex)
    for a in range(4):
        ia = np.clip(u0.astype(int) - 1 + a, 0, G - 1)
        for b in range(4):
            ib = np.clip(v0.astype(int) - 1 + b, 0, G - 1)
            out += wu[:, a] * wv[:, b] * F[ia, ib]
    return out
