"""Training of the learned preconditioner on solutions of the plain solver.

Data: `scatterers` random scatterers (kappa ~ U[kappa_lo, kappa_hi]; 1 to 4
Gaussian bumps with centres U[-0.6, 0.6]^2, amplitudes U[0.5, 1.5] and widths
U[0.05, 0.2]; all seeded), each assembled on a uniform tree and solved by the
batched mixed-precision solver (ls_gmres_mixed_batched) for right-hand sides
f = -kappa^2 q u of two kinds: `angles` plane-wave incidences
u = exp(i kappa d_m . x), d_m at theta_m = 2 pi m / angles, and `off_shell`
waves u = exp(i (k . x + psi)) with |k| ~ kappa U[0.25, 2], random direction
and phase. The second kind stands in for the residual-like vectors that a
preconditioner is applied to inside GMRES, which are not incident fields.
Right-hand sides f and the multiple-scattering parts phi - f of their
solutions are resampled to the network's grid with the Chebyshev-Q+
interpolation (ls_op_grid_sample); the network learns f -> phi - f.

Training samples are random complex superpositions of one scatterer's
(f, phi) pairs - exact solutions by linearity - scaled to unit RMS and built
on the GPU (ls_fno_make_batch). Loss, gradients and Adam steps run in the
network's own CUDA kernels (ls_fno_loss_grad, ls_fno_adam_step). torch only
holds device buffers.

    python -m lippmann_schwinger_solver_gb300.fno_train --out weights.lsfno
"""
import argparse
import json
import math
import time

import numpy as np

from . import (FNO, FNO_KAPPA_SCALE, Config, Operator)


def scatterer(rng, kappa_lo=10.0, kappa_hi=40.0):
    """kappa and bumps of one random scatterer."""
    kappa = float(rng.uniform(kappa_lo, kappa_hi))
    n = int(rng.integers(1, 5))
    bumps = [(float(rng.uniform(-0.6, 0.6)), float(rng.uniform(-0.6, 0.6)), float(rng.uniform(0.5, 1.5)),
              float(rng.uniform(0.05, 0.2))) for _ in range(n)]
    return kappa, bumps


def operator_config(kappa, bumps, level, tol_pow):
    return Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=tol_pow, degreeOfBases=6, nLevelsUniform=level,
                  Qchoice=6, findPhi=1, reference_rounding=0, L=1.0, kappa=kappa, bumps=bumps)


def off_shell_rhs(op, kappa, n, rng):
    """-kappa^2 q exp(i (k . x + psi)) for n random wave vectors with
    |k| = kappa U[0.25, 2] (N x n)."""
    xy = op.points()
    q = op.contrast()
    mag = kappa * rng.uniform(0.25, 2.0, n)
    ang = rng.uniform(0, 2 * np.pi, n)
    psi = rng.uniform(0, 2 * np.pi, n)
    phase = np.outer(xy[:, 0], mag * np.cos(ang)) + np.outer(xy[:, 1], mag * np.sin(ang)) + psi
    return np.asfortranarray(-(kappa * kappa) * q[:, None] * np.exp(1j * phase))


def generate(n_scatterers, angles, level, grid, seed, tol=1e-6, tol_pow=8, kappa_lo=10.0, kappa_hi=40.0,
             off_shell=0, device=0, log=print):
    """Solves the scatterers and returns the grid data on the GPU (torch
    tensors): F (right-hand sides) and PHI (phi - f) [S, angles + off_shell,
    G*G] complex64 (plane waves first), Q [S, G*G], KAP [S] (kappa / 40),
    and per-scatterer records."""
    import torch
    dev = torch.device("cuda", device)
    rng = np.random.default_rng(seed)
    GG = grid * grid
    nb = angles + off_shell
    F = torch.empty((n_scatterers, nb, GG), dtype=torch.complex64, device=dev)
    PHI = torch.empty_like(F)
    Q = torch.empty((n_scatterers, GG), dtype=torch.float32, device=dev)
    KAP = torch.empty(n_scatterers, dtype=torch.float32, device=dev)
    thetas = 2 * np.pi * np.arange(angles) / angles
    recs = []
    for s in range(n_scatterers):
        kappa, bumps = scatterer(rng, kappa_lo, kappa_hi)
        t0 = time.time()
        op = Operator(operator_config(kappa, bumps, level, tol_pow), device=device)
        op.enable_f32()
        t1 = time.time()
        B = op.rhs_angles(thetas)
        if off_shell:
            B = np.asfortranarray(np.concatenate([B, off_shell_rhs(op, kappa, off_shell, rng)], axis=1))
        X, nmv, rr, code = op.gmres_mixed_batched(B, max_outer=10, inner_iter=100, tol=tol)
        t2 = time.time()
        b_dev = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
        x_dev = torch.from_numpy(np.ascontiguousarray((X - B).T)).to(dev)
        st = torch.cuda.current_stream(dev).cuda_stream
        op.grid_sample_device(grid, nb, b_dev.data_ptr(), F[s].data_ptr(), stream=st)
        op.grid_sample_device(grid, nb, x_dev.data_ptr(), PHI[s].data_ptr(), stream=st)
        Q[s] = torch.from_numpy(op.grid_contrast(grid)).to(dev)
        KAP[s] = kappa / FNO_KAPPA_SCALE
        torch.cuda.synchronize(dev)
        recs.append(dict(kappa=kappa, bumps=len(bumps), N=op.N, assemble_s=round(t1 - t0, 2),
                         solve_s=round(t2 - t1, 3), max_residual=float(np.max(rr)), status=int(code)))
        log(json.dumps(dict(scatterer=s, **recs[-1])))
        op.close()
    return dict(F=F, PHI=PHI, Q=Q, KAP=KAP, records=recs, angles=angles, off_shell=off_shell)


def train(net, data, steps, batch=16, lr=1e-3, seed=1, log_every=100, log=print, train_scatterers=None):
    """Adam on random superpositions; cosine learning-rate decay to lr/20.
    Returns the loss history (one value per log_every steps)."""
    import torch
    F, PHI, Q, KAP = data["F"], data["PHI"], data["Q"], data["KAP"]
    dev = F.device
    S, nb, GG = F.shape
    idx = np.arange(S) if train_scatterers is None else np.asarray(train_scatterers)
    rng = np.random.default_rng(seed)
    inp = torch.empty((batch, GG, 6), dtype=torch.float32, device=dev)
    tgt = torch.empty((batch, GG, 2), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    hist = []
    t0 = time.time()
    for step in range(steps):
        sidx = rng.choice(idx, size=batch).astype(np.int32)
        # Half of the samples are single incidences, half dense superpositions.
        coef = np.zeros((batch, nb), dtype=np.complex64)
        for b in range(batch):
            if b % 2 == 0:
                coef[b, rng.integers(nb)] = np.exp(2j * np.pi * rng.uniform())
            else:
                coef[b] = (rng.standard_normal(nb) + 1j * rng.standard_normal(nb)) / np.sqrt(2 * nb)
        s_dev = torch.from_numpy(sidx).to(dev)
        c_dev = torch.from_numpy(coef).to(dev)
        net.make_batch_device(batch, nb, S, F.data_ptr(), PHI.data_ptr(), Q.data_ptr(), KAP.data_ptr(),
                              s_dev.data_ptr(), c_dev.data_ptr(), inp.data_ptr(), tgt.data_ptr(), stream=st)
        want = (step % log_every == 0) or step == steps - 1
        loss = net.loss_grad_device(batch, inp.data_ptr(), tgt.data_ptr(), want_loss=want, stream=st)
        a = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * step / steps)))
        net.adam_step(a, stream=st)
        if want:
            hist.append((step, loss))
            log(json.dumps(dict(step=step, loss=loss, lr=a, seconds=round(time.time() - t0, 1))))
    torch.cuda.synchronize(dev)
    return hist


def evaluate(net, data, scatterers, batch=16, columns=None):
    """Mean relative L2 error of f + net(f) against the solution phi on
    single right-hand sides of the given scatterers (grid values); columns:
    which of them (default the plane waves)."""
    import torch
    F, PHI, Q, KAP = data["F"], data["PHI"], data["Q"], data["KAP"]
    dev = F.device
    S, nb, GG = F.shape
    cols = list(range(data.get("angles", nb))) if columns is None else list(columns)
    inp = torch.empty((batch, GG, 6), dtype=torch.float32, device=dev)
    tgt = torch.empty((batch, GG, 2), dtype=torch.float32, device=dev)
    out = torch.empty((batch, GG, 2), dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    errs = []
    for s in scatterers:
        for m0 in range(0, len(cols), batch):
            ms = cols[m0:m0 + batch]
            coef = np.zeros((len(ms), nb), dtype=np.complex64)
            for i, m in enumerate(ms):
                coef[i, m] = 1.0
            sidx = np.full(len(ms), s, dtype=np.int32)
            s_dev = torch.from_numpy(sidx).to(dev)
            c_dev = torch.from_numpy(coef).to(dev)
            net.make_batch_device(len(ms), nb, S, F.data_ptr(), PHI.data_ptr(), Q.data_ptr(), KAP.data_ptr(),
                                  s_dev.data_ptr(), c_dev.data_ptr(), inp.data_ptr(), tgt.data_ptr(), stream=st)
            net.forward_device(len(ms), inp.data_ptr(), out.data_ptr(), stream=st)
            torch.cuda.synchronize(dev)
            o = out[:len(ms)].double()
            t = tgt[:len(ms)].double()
            phi = t + inp[:len(ms), :, 1:3].double()
            e = ((o - t) ** 2).sum(dim=(1, 2)).sqrt() / (phi ** 2).sum(dim=(1, 2)).sqrt()
            errs += e.cpu().tolist()
    return float(np.mean(errs))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--scatterers", type=int, default=64)
    ap.add_argument("--held-out", type=int, default=4, help="scatterers kept out of training, for evaluation")
    ap.add_argument("--angles", type=int, default=32)
    ap.add_argument("--off-shell", type=int, default=32)
    ap.add_argument("--level", type=int, default=4)
    ap.add_argument("--tol-pow", type=int, default=8)
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--modes", type=int, default=24)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--proj-width", type=int, default=128)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--out", required=True)
    ap.add_argument("--f32", action="store_true", help="store float32 weights (default float16)")
    a = ap.parse_args(argv)
    data = generate(a.scatterers, a.angles, a.level, a.grid, a.seed, tol_pow=a.tol_pow, off_shell=a.off_shell)
    net = FNO(grid=a.grid, modes=a.modes, layers=a.layers, proj_width=a.proj_width, seed=a.seed)
    n_train = a.scatterers - a.held_out
    before = evaluate(net, data, range(n_train, a.scatterers))
    t0 = time.time()
    hist = train(net, data, a.steps, batch=a.batch, lr=a.lr, seed=a.seed + 1, train_scatterers=range(n_train))
    secs = time.time() - t0
    after_train = evaluate(net, data, range(min(4, n_train)))
    after = evaluate(net, data, range(n_train, a.scatterers))
    after_off = evaluate(net, data, range(n_train, a.scatterers), columns=range(a.angles, a.angles + a.off_shell))
    net.save(a.out, half=not a.f32)
    print(json.dumps(dict(train_seconds=round(secs, 1), steps=a.steps, batch=a.batch, final_loss=hist[-1][1],
                          heldout_rel_err_before=before, heldout_rel_err_after=after,
                          heldout_off_shell_rel_err_after=after_off, train_rel_err_after=after_train,
                          solutions=a.scatterers * (a.angles + a.off_shell), weights=a.out)))


if __name__ == "__main__":
    main()
