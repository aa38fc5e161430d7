"""Many scatterers, many incidence directions (the batched workload).

Each scatterer (uniform tree of level 4-6, kappa ~ U[10, 60], 1 to 4
Gaussian bumps with centres U[-0.6, 0.6]^2, amplitudes U[0.5, 1.5], widths
U[0.05, 0.2], all seeded) is assembled on the host, uploaded, and solved for
`angles` plane-wave incidences theta_m = 2 pi m / angles by the batched
mixed-precision solver (ls_gmres_mixed_batched: 64 directions per FP32
operator apply on the tensor cores, FP64 true residual per direction). The host assembly of the
next scatterer runs in a second thread while the GPU solves the current one:
ctypes releases the interpreter lock during each library call.

    python -m lippmann_schwinger_solver_gb300.scatterers --n 32 --angles 64
"""
import argparse
import json
import threading
import time

import numpy as np

from . import Config, LS_OK, Operator


def scatterer_specs(n, seed, levels=(4, 5, 6), kappa_lo=10.0, kappa_hi=60.0):
    """n seeded scatterers: (level, kappa, bumps)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        level = int(rng.choice(levels))
        kappa = float(rng.uniform(kappa_lo, kappa_hi))
        nb = int(rng.integers(1, 5))
        bumps = tuple((float(rng.uniform(-0.6, 0.6)), float(rng.uniform(-0.6, 0.6)), float(rng.uniform(0.5, 1.5)),
                       float(rng.uniform(0.05, 0.2))) for _ in range(nb))
        out.append((level, kappa, bumps))
    return out


def config(level, kappa, bumps, tol_pow=10, precompute_on_gpu=0, far_on_gpu=0):
    return Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=tol_pow, degreeOfBases=6, nLevelsUniform=level,
                  Qchoice=6, findPhi=1, reference_rounding=1, L=1.0, kappa=kappa, bumps=bumps,
                  precompute_on_gpu=precompute_on_gpu, far_on_gpu=far_on_gpu)


def solve_many(specs, angles=64, tol=1e-8, tol_pow=10, device=0, log=None, keep_solutions=False,
               precompute_on_gpu=0, far_on_gpu=0, workers=1):
    """Assembles and solves every scatterer; returns per-scatterer records and
    the totals. With precompute_on_gpu the precomputation quadratures run on
    the GPU, with far_on_gpu the far-field table (1), NCA (2) and M2L block
    fill (3) (see ls_config).
    workers = 1: the assembly of scatterer k + 1 overlaps the solve of k.
    workers = W > 1: a work queue in scatterer order; W threads assemble
    (at most 2W operators built and not yet solved) and W threads solve, each
    on its own operator's streams, so small solves share the GPU.
    assemble_s is the operator's creation (host assembly, upload, FP32
    copy); host_stages_s splits the host assembly by stage."""
    thetas = 2 * np.pi * np.arange(angles) / angles
    n = len(specs)

    def create(k):
        t0 = time.perf_counter()
        op = Operator(config(*specs[k], tol_pow=tol_pow, precompute_on_gpu=precompute_on_gpu,
                             far_on_gpu=far_on_gpu), device=device)
        op.enable_f32()
        return op, time.perf_counter() - t0

    def solve(k, op, t_asm):
        level, kappa, bumps = specs[k]
        B = op.rhs_angles(thetas)
        t0 = time.perf_counter()
        X, nmv, rr, code = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=tol)
        t_solve = time.perf_counter() - t0
        rec = dict(scatterer=k, level=level, kappa=round(kappa, 3), bumps=len(bumps), N=op.N,
                   assemble_s=round(t_asm, 3),
                   host_stages_s=dict(zip(("geometry", "precompute", "lists", "nca", "checks", "pack"),
                                          (round(t, 3) for t in op.info["assemble_stage_seconds"]))),
                   solve_s=round(t_solve, 4), applies_and_fp64_products=nmv,
                   max_true_residual=float(np.max(rr)), converged=code == LS_OK)
        if log:
            log(json.dumps(rec))
        op.close()
        return rec, (X if keep_solutions else None)

    t_start = time.perf_counter()
    if workers <= 1:
        out = []
        ready = {}

        def build(k):
            try:
                ready[k] = create(k) + (None,)
            except Exception as e:  # reported with the scatterer, not raised from the thread
                ready[k] = (None, 0.0, e)

        th = threading.Thread(target=build, args=(0,))
        th.start()
        for k in range(n):
            th.join()
            op, t_asm, err = ready.pop(k)
            if k + 1 < n:
                th = threading.Thread(target=build, args=(k + 1,))
                th.start()
            if err is not None:
                raise err
            out.append(solve(k, op, t_asm))
    else:
        from concurrent.futures import ThreadPoolExecutor
        slots = threading.Semaphore(2 * workers)
        stop = threading.Event()
        taken = set()

        def build_q(k):
            while not slots.acquire(timeout=0.05):
                if stop.is_set():
                    raise RuntimeError("stopped")
            try:
                if stop.is_set():
                    raise RuntimeError("stopped")
                return create(k)
            except BaseException:
                slots.release()
                raise

        def solve_q(k):
            op, t_asm = futs[k].result()
            taken.add(k)
            try:
                return solve(k, op, t_asm)
            finally:
                slots.release()

        with ThreadPoolExecutor(workers) as builders, ThreadPoolExecutor(workers) as solvers:
            futs = [builders.submit(build_q, k) for k in range(n)]
            try:
                out = list(solvers.map(solve_q, range(n)))
            except BaseException:
                # A scatterer failed: stop the queue and free the operators
                # that were built and not taken by a solver.
                stop.set()
                for f in futs:
                    f.cancel()
                for k, f in enumerate(futs):
                    if k not in taken and f.done() and not f.cancelled() and f.exception() is None:
                        f.result()[0].close()
                raise
    wall = time.perf_counter() - t_start
    recs = [r for r, _ in out]
    sols = [x for _, x in out] if keep_solutions else []
    total = dict(scatterers=n, directions=angles, solutions=n * angles, tol=tol, workers=workers,
                 wall_s=round(wall, 2), assemble_s=round(sum(r["assemble_s"] for r in recs), 2),
                 solve_s=round(sum(r["solve_s"] for r in recs), 3),
                 solve_per_direction_ms=round(1e3 * sum(r["solve_s"] for r in recs) / (n * angles), 3),
                 all_converged=all(r["converged"] for r in recs),
                 max_true_residual=max(r["max_true_residual"] for r in recs))
    return recs, total, sols


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--angles", type=int, default=64)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--tol-pow", type=int, default=10)
    ap.add_argument("--levels", default="4,5,6")
    ap.add_argument("--gpu-precompute", action="store_true", help="precomputation quadratures on the GPU")
    ap.add_argument("--gpu-far", type=int, default=0, choices=[0, 1, 2, 3],
                    help="far-field table (1), NCA skeleton search (2) and M2L block fill (3) on the GPU")
    ap.add_argument("--workers", type=int, default=1,
                    help="scatterers assembled and solved at once (a work queue when > 1)")
    a = ap.parse_args(argv)
    specs = scatterer_specs(a.n, a.seed, levels=tuple(int(v) for v in a.levels.split(",")))
    _, total, _ = solve_many(specs, a.angles, a.tol, a.tol_pow, log=print, precompute_on_gpu=int(a.gpu_precompute),
                             far_on_gpu=a.gpu_far, workers=a.workers)
    print(json.dumps(total))


if __name__ == "__main__":
    main()
