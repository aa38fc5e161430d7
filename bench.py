"""Benchmark: FP64 DAFMM matvec throughput (matvec/s) on one GB300.

Workload (the reference's scale configuration): uniform quadtree level 6
(4,096 leaves, 6x6 Chebyshev nodes, N = 147,456), kappa = 40, contrast =
3 Gaussian bumps drawn from numpy.random.default_rng(20261203) (centres
U[-0.6,0.6]^2, amplitudes U[0.5,1.5], widths U[0.05,0.2]), NCA tolerance
1e-10, 16 cones at the finest HFR level, degree-6 basis, 6-digit
precomputation rounding as in the reference. One step = one matvec y = A x
of the assembled operator over one synthetic input vector (re, im ~ U[-1,1]).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference algorithm
(oracle/, all host threads) on the same workload; the reference itself needs
Eigen and Boost.Math, which are not installed, so its own build is
unavailable. N > 1 runs independent replicas (the path has no data-path
collective), one per GPU, and reports the sum of their throughputs.
"""
import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DAFMM matvec throughput, FP64 (plain method), N=147456, kappa=40"
SEED = 20261203


FNO_WEIGHTS = os.path.join(ROOT, "lippmann_schwinger_solver_gb300", "weights", "fno_k10_40.lsfno")


def workload_config(ls, level=6):
    return ls.Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=10, degreeOfBases=6, nLevelsUniform=level,
                     Qchoice=6, findPhi=1, reference_rounding=1, L=1.0, kappa=40.0, bumps=ls.seeded_bumps(SEED))


def input_vector(n):
    rng = np.random.default_rng(SEED + 1)
    return rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)


def traffic_per_launch(kernels):
    """DRAM bytes of one M2L launch at the benchmark size, from the ncu capture
    summarised in profiles/ (None when absent)."""
    tp = os.path.join(ROOT, "profiles", "m2l_traffic.json")
    if not os.path.exists(tp):
        return None
    with open(tp) as f:
        return json.load(f).get(kernels, {}).get("bytes_per_launch")


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(value, dist, device=None):
    """The slowest rank's value (timings of replicas are reported as the max
    over ranks, so that whole-job throughput = ranks * steps / max time)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, ms_per_step):
    """Whole-job matvec/s of `world` independent replicas whose slowest
    step takes ms_per_step."""
    return world * 1e3 / ms_per_step


def cpu_model():
    """The host CPU's model name (lscpu), or the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform

    return platform.machine()


def _timed_matvecs(o, x, budget_s, cap):
    """matvec/s of the oracle: as many matvecs as fit in budget_s (>= 1)."""
    n, t = 0, 0.0
    while n < 1 or (t < budget_s and n < cap):
        t1 = time.perf_counter()
        o.matvec(x)
        t += time.perf_counter() - t1
        n += 1
    return n / t, n


def c1_config(ls):
    """The reference's CPU-runnable configuration: uniform level 4 (N=9,216),
    kappa 10, Gaussian contrast 1.5 exp(-160|x|^2), NCA tolerance 1e-8."""
    return ls.Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=4,
                     Qchoice=0, findPhi=1, reference_rounding=1, L=1.0, kappa=10.0)


def readme_adaptive_config(ls):
    """The reference's published run (GMRES/Readme.md:43): adaptive quadtree
    (tolerance 1e-5, 5 levels, N=5,328), nCones_LFR 16, 6x6 nodes, L = 0.5,
    kappa 40, NCA tolerance 1e-8, Gaussian contrast."""
    return ls.Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=8, degreeOfBases=6, nLevelsUniform=5,
                     Qchoice=0, findPhi=1, reference_rounding=1, L=0.5, kappa=40.0, tree_adaptive=1,
                     treeAdaptivity=5)


# Residuals the reference prints for RestartedGMRES(m = 10) after 1 and 2
# restarts at that configuration (GMRES/Readme.md:64-65, 84-85).
README_RESIDUALS = {1: 4.59412e-06, 2: 1.28443e-10}


def _device_matvec_ms(op, iters, warmup):
    """Mean time of back-to-back FP64 matvecs with device-resident x on
    torch's current stream (CUDA events around the whole loop)."""
    import torch
    x = torch.from_numpy(input_vector(op.N)).cuda()
    y = torch.empty_like(x)
    st = torch.cuda.current_stream().cuda_stream
    for _ in range(warmup):
        op.matvec_device(x.data_ptr(), y.data_ptr(), st)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(iters):
        op.matvec_device(x.data_ptr(), y.data_ptr(), st)
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / iters


def adaptive_leg(ls, local, timed, max_iter):
    """The adaptive operator at the README configuration: matvec time,
    RestartedGMRES(10) with 1 and 2 restarts against the published
    residuals, and the solves to 1e-8."""
    opa = ls.Operator(readme_adaptive_config(ls), device=local)
    info = opa.info
    ms_a = _device_matvec_ms(opa, 200, 5)
    ba = opa.rhs()
    out = {"config": "adaptive quadtree (GMRES/Readme.md:43), N=%d, %d levels" % (opa.N, info["n_levels"]),
           "N": opa.N, "assemble_s": info["assemble_seconds"],
           "assemble_stages_s": dict(zip(("geometry", "precompute", "lists", "nca", "checks", "pack"),
                                         (round(t, 3) for t in info["assemble_stage_seconds"]))),
           "far_entries": info["far_entries"], "near_entries": info["near_entries"],
           "matvec_ms": ms_a, "matvec_per_s": 1e3 / ms_a, "restarted_gmres_m10": {}}
    # The same tree with the precomputation quadratures on the GPU.
    opg = ls.Operator(dataclasses.replace(readme_adaptive_config(ls), precompute_on_gpu=1), device=local)
    xr = input_vector(opa.N)
    yh = opa.matvec(xr)
    out["gpu_precompute"] = {"assemble_s": opg.info["assemble_seconds"],
                             "precompute_s": opg.info["assemble_stage_seconds"][1],
                             "host_precompute_s": info["assemble_stage_seconds"][1],
                             "matvec_rel_diff_vs_host_integrated": float(np.linalg.norm(opg.matvec(xr) - yh) /
                                                                         np.linalg.norm(yh))}
    opg.close()
    nb = np.linalg.norm(ba)
    for restarts, published in README_RESIDUALS.items():
        t, xr = timed(lambda: opa.gmres_restarted(ba, 10, restarts))
        res = float(np.linalg.norm(ba - opa.matvec(xr)) / nb)
        out["restarted_gmres_m10"][str(restarts)] = {"s": t, "residual": res, "published": published,
                                                     "rel_diff": abs(res / published - 1.0)}
    t64, (x64, _, it64, rr64, code64) = timed(lambda: opa.gmres(ba, max_iter=max_iter, tol=1e-8))
    opa.enable_f32()
    tm, (xm, _, nmv, rrm, codem) = timed(lambda: opa.gmres_mixed(ba, max_outer=20, inner_iter=max_iter, tol=1e-8))
    out.update({"fp64_gmres_s": t64, "fp64_iters": it64, "fp64_true_residual": rr64, "fp64_converged": code64 == 0,
                "mixed_s": tm, "mixed_matvecs": nmv, "mixed_true_residual": rrm, "mixed_converged": codem == 0,
                "mixed_rel_err_vs_fp64": float(np.linalg.norm(xm - x64) / np.linalg.norm(x64))})
    opa.close()
    return out


def gpu_assembly_leg(ls, cfg, x, y_host, skel_host, device):
    """The workload's operator assembled with its far field on the GPU
    (ls_config.far_on_gpu 1: sum table; 2: table and NCA; 3: and the M2L
    tiles filled on the device; then also the precomputation quadratures)
    against the default host-assembled one,
    which the oracle leg pins: assembly stages, the matvec's distance and
    the fraction of skeleton nodes that agree."""
    names = ("geometry", "precompute", "lists", "nca", "checks", "pack")
    out = {"tolerance": 10.0 ** (1 - cfg.TOL_POW)}
    for name, over in (("far_table", dict(far_on_gpu=1)), ("far_table_and_nca", dict(far_on_gpu=2)),
                       ("far_table_nca_and_m2l_fill", dict(far_on_gpu=3)),
                       ("far_and_precompute", dict(far_on_gpu=3, precompute_on_gpu=1))):
        t0 = time.perf_counter()
        opg = ls.Operator(dataclasses.replace(cfg, **over), device=device)
        wall = time.perf_counter() - t0
        y = opg.matvec(x)
        ig = opg.info
        out[name] = {"assemble_s": ig["assemble_seconds"], "operator_create_s": wall,
                     "assemble_stages_s": dict(zip(names, (round(t, 3) for t in ig["assemble_stage_seconds"]))),
                     "rel_l2_vs_host_operator": float(np.linalg.norm(y - y_host) / np.linalg.norm(y_host)),
                     "skeleton_nodes_equal": ls.skeleton_agreement(opg.skeleton_dump(), skel_host),
                     "max_rank": ig["max_rank"]}
        opg.close()
    return out


def oracle_leg(ls, cfg, y_gpu, skel_gpu, budget_s=20.0):
    """The CPU restatement of the reference (oracle/) on the machine's host cores:
    its matvec/s with all threads and with one, its GMRES solve time to a
    relative residual of 1e-8 at this workload and at the 9,216-point C1
    configuration, and the GPU product's parity with it on the same input
    (relative L2 distance and skeleton equality)."""
    from oracle import oracle as ora

    ora.build()
    ncores = os.cpu_count() or 1
    ora.set_threads(ncores)
    t0 = time.time()
    o = ora.Oracle(cfg.as_dict())
    t_asm = time.time() - t0
    x = input_vector(o.N)
    yo = o.matvec(x)  # also the warm-up
    parity = {"rel_l2_vs_oracle": float(np.linalg.norm(y_gpu - yo) / np.linalg.norm(yo)),
              "skeletons_equal": bool(np.array_equal(skel_gpu, o.skeleton_dump())),
              "tolerance": 1e-10, "input": "seeded x (re, im ~ U[-1,1], seed %d)" % (SEED + 1)}
    v_all, n_all = _timed_matvecs(o, x, budget_s, 200)
    ora.set_threads(1)
    v_one, n_one = _timed_matvecs(o, x, min(6.0, budget_s), 50)
    ora.set_threads(ncores)
    b = o.rhs()
    t1 = time.perf_counter()
    xs, hist, it = o.gmres(b, max_iter=400, tol=1e-8)
    t_solve = time.perf_counter() - t1
    rr = float(np.linalg.norm(b - o.matvec(xs)) / np.linalg.norm(b))
    o.close()
    o1 = ora.Oracle(c1_config(ls).as_dict())
    b1 = o1.rhs()
    t1 = time.perf_counter()
    x1, _, it1 = o1.gmres(b1, max_iter=400, tol=1e-8)
    t_solve1 = time.perf_counter() - t1
    rr1 = float(np.linalg.norm(b1 - o1.matvec(x1)) / np.linalg.norm(b1))
    o1.close()
    cpu = {"value": v_all, "unit": "matvec/s", "cores": ncores, "kind": "port", "cpu_model": cpu_model(),
           "sample": f"{n_all} oracle matvecs of the full workload operator with {ncores} threads, {n_one} with 1 "
                     f"(assembly {t_asm:.0f} s not timed)",
           "one_thread": {"value": v_one, "unit": "matvec/s", "cores": 1},
           "solve_s": {"workload": t_solve, "workload_iters": it, "workload_true_residual": rr,
                       "c1": t_solve1, "c1_iters": it1, "c1_true_residual": rr1, "tol": 1e-8,
                       "method": "oracle GMRES (x0 = 0, Givens residual estimate), all threads"}}
    return cpu, parity


def run_reference(args):
    """The CPU arm: the oracle restatement of the reference, all host threads."""
    import lippmann_schwinger_solver_gb300 as ls

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cfg = workload_config(ls, args.level)
    from oracle import oracle as ora

    ora.build()
    ncores = os.cpu_count() or 1
    ora.set_threads(ncores)
    o = ora.Oracle(cfg.as_dict())
    x = input_vector(o.N)
    warmup = max(1, args.warmup)
    for _ in range(warmup):
        o.matvec(x)
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.matvec(x)
    dt = time.perf_counter() - t0
    v = steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "matvec/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (f64)", "data": "synthetic",
            "config": {"workload": "uniform level %d, N=%d, kappa=40, 3 seeded bumps (seed %d), NCA tol 1e-10"
                                   % (args.level, o.N, SEED), "parallelism": "CPU threads"},
            "cpu_baseline": {"value": v, "unit": "matvec/s", "cores": ncores, "kind": "port", "cpu_model": cpu_model(),
                             "sample": f"{steps} matvecs of the full workload operator after {warmup} warm-ups; "
                                       "reference build unavailable (Eigen/Boost headers missing)"},
            "e2e": {"value": v, "unit": "matvec/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    import lippmann_schwinger_solver_gb300 as ls

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    ls.build()
    cfg = workload_config(ls, args.level)
    op = ls.Operator(cfg, device=local)
    info = op.info
    n = op.N
    x = input_vector(n)
    xd = torch.from_numpy(x).to(f"cuda:{local}")
    yd = torch.empty_like(xd)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    prec = ls.LS_PREC_F32 if args.precision == "f32" else ls.LS_PREC_F64
    if prec == ls.LS_PREC_F32:
        op.enable_f32()
    df_kernels = args.f64_kernels == "double-float"
    if df_kernels:
        op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT)
        info = op._info()  # launch count of the selected kernels
    # warm-up
    for _ in range(max(3, args.warmup)):
        op.matvec_device(xd.data_ptr(), yd.data_ptr(), sp, precision=prec)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        ev0.record(stream)
        for _ in range(args.steps):
            op.matvec_device(xd.data_ptr(), yd.data_ptr(), sp, precision=prec)
        ev1.record(stream)
        torch.cuda.synchronize()
        time.sleep(0.3)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, dist, f"cuda:{local}")
    value = replica_throughput(world, ms)
    # Dominant kernel (M2L) timed with events on the operator's own stream.
    ms_mv, ms_m2l = op.time_matvec(warmup=3, iters=max(5, args.steps), precision=prec)
    if prec == ls.LS_PREC_F32:
        # Profiling / reference run of the FP32 operator: one JSON line, no e2e.
        print(json.dumps({"metric": "DAFMM matvec throughput, FP32 operator", "value": world * 1e3 / ms,
                          "unit": "matvec/s", "ms_per_step": ms, "m2l_ms": ms_m2l, "n_gpus": world}), flush=True)
        op.close()
        return
    # End to end through the C ABI with host buffers (pinned).
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    lib = ls.lib()
    import ctypes

    xp = ctypes.cast(xh.data_ptr(), ctypes.POINTER(ctypes.c_double))
    yp = ctypes.cast(yh.data_ptr(), ctypes.POINTER(ctypes.c_double))
    for _ in range(2):
        lib.ls_matvec_host(op._h, xp, yp)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc = lib.ls_matvec_host(op._h, xp, yp)
        if rc != 0:
            raise RuntimeError(lib.ls_last_error().decode())
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, dist, f"cuda:{local}")
    # The bench output must agree with the C ABI host path bit for bit.
    assert np.array_equal(yh.numpy(), yd.cpu().numpy()), "device and host-buffer matvecs differ"
    # The other kernel choice behind the FP64 entry points on the same
    # operator and input: its speed and its distance from the timed product.
    other = ls.LS_F64_NATIVE if df_kernels else ls.LS_F64_DOUBLE_FLOAT
    op.set_f64_kernels(other)
    ms_o, m2l_o = op.time_matvec(warmup=3, iters=max(5, args.steps), precision=ls.LS_PREC_F64)
    yo = torch.empty_like(xd)
    op.matvec_device(xd.data_ptr(), yo.data_ptr(), sp)
    torch.cuda.synchronize()
    y_main = yd.cpu().numpy()
    other_name = "native" if other == ls.LS_F64_NATIVE else "double-float"
    peak_o, peak_kind_o = load_peaks()
    achieved_o = info["m2l_bytes"] / (m2l_o * 1e-3) / 1e9
    alt = {"f64_kernels": other_name,
           "matvec_per_s": 1e3 / ms_o, "ms_per_step": ms_o, "m2l_ms": m2l_o,
           "roofline": {"bound": "hbm", "achieved": achieved_o, "peak": peak_o, "unit": "GB/s",
                        "frac": achieved_o / peak_o, "traffic": traffic_per_launch(other_name),
                        "peak_source": peak_kind_o,
                        "kernel": "gemv_df_kernel<1> (M2L)" if other_name == "double-float"
                        else "gemv_tiles_kernel<double2, 1> (M2L)"},
           "rel_l2_vs_timed": float(np.linalg.norm(yo.cpu().numpy() - y_main) / np.linalg.norm(y_main))}
    op.set_f64_kernels(ls.LS_F64_DOUBLE_FLOAT if df_kernels else ls.LS_F64_NATIVE)
    # Solve time to a true relative residual of 1e-8: plain FP64 GMRES, and
    # the FP64 refinement around the FP32 operator (residual always FP64).
    solve = None
    if not args.no_solve:
        b = op.rhs()

        def timed(fn):
            fn()  # first call: workspaces, preconditioner set-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = fn()
            return time.perf_counter() - t0, r
        t64, (x64, hist64, it64, rr64, code64) = timed(lambda: op.gmres(b, max_iter=args.max_iter, tol=1e-8))
        op.enable_f32()
        ms32, m2l32 = op.time_matvec(warmup=3, iters=max(5, args.steps), precision=ls.LS_PREC_F32)
        tm, (xm, histm, nmv, rrm, codem) = timed(
            lambda: op.gmres_mixed(b, max_outer=20, inner_iter=args.max_iter, tol=1e-8))

        def err_vs_fp64(xv):
            return float(np.linalg.norm(xv - x64) / np.linalg.norm(x64))
        solve = {"tol": 1e-8, "fp64_gmres_s": t64, "fp64_iters": it64, "fp64_true_residual": rr64,
                 "fp64_converged": code64 == 0, "fp64_history": [float(v) for v in hist64],
                 "mixed_s": tm, "mixed_matvecs": nmv, "mixed_true_residual": rrm,
                 "mixed_converged": codem == 0, "speedup_mixed_vs_fp64": t64 / tm if tm > 0 else None,
                 "mixed_rel_err_vs_fp64": err_vs_fp64(xm), "mixed_history": [float(v) for v in histm],
                 "f32_matvec_per_s": 1e3 / ms32, "f32_m2l_ms": m2l32}
        # The same refinement with the inner Krylov basis and its Gram-Schmidt
        # in FP32 (the default above keeps them in FP64).
        op.set_inner_basis(ls.LS_INNER_BASIS_F32)
        tm32, (xm32, histm32, nmv32, rrm32, codem32) = timed(
            lambda: op.gmres_mixed(b, max_outer=20, inner_iter=args.max_iter, tol=1e-8))
        op.set_inner_basis(ls.LS_INNER_BASIS_F64)
        solve["mixed_inner_basis"] = "fp64"
        solve["mixed_fp32_basis"] = {"s": tm32, "matvecs": nmv32, "true_residual": rrm32, "converged": codem32 == 0,
                                     "rel_err_vs_fp64": err_vs_fp64(xm32), "speedup_vs_fp64": t64 / tm32,
                                     "history": [float(v) for v in histm32]}
        # The same solves at the 9,216-point C1 configuration (GPU side of the
        # CPU solve times in cpu_baseline.solve_s).
        op1 = ls.Operator(c1_config(ls), device=local)
        b1 = op1.rhs()
        t64_1, (_, _, it64_1, rr64_1, _) = timed(lambda: op1.gmres(b1, max_iter=args.max_iter, tol=1e-8))
        solve["c1"] = {"fp64_gmres_s": t64_1, "fp64_iters": it64_1, "fp64_true_residual": rr64_1, "N": op1.N}
        op1.close()
        # The learned preconditioner: mixed-precision flexible GMRES with the
        # trained spectral neural operator as initial guess and right
        # preconditioner (the NN-FGMRES leg of the solve-time metric).
        if not args.no_nn and os.path.exists(FNO_WEIGHTS):
            net = ls.FNO.load(FNO_WEIGHTS, device=local)
            nn = {"weights": os.path.relpath(FNO_WEIGHTS, ROOT), "params": net.n_params}
            for name, flags in (("nn", ls.LS_NN_GUESS | ls.LS_NN_PRECOND), ("nn_guess_only", ls.LS_NN_GUESS),
                                ("nn_precond_only", ls.LS_NN_PRECOND)):
                tn, (xn, hn, rep, coden) = timed(
                    lambda: op.fgmres_nn(net, b, flags=flags, max_outer=20, inner_iter=args.max_iter, tol=1e-8))
                nn[name] = {"s": tn, "converged": coden == 0, "true_residual": rep["rel_residual"],
                            "rel_err_vs_fp64": err_vs_fp64(xn),
                            "fp32_applies_and_fp64_products": rep["n_matvec"], "network_applies": rep["n_precond"],
                            "guess_residual": rep["guess_residual"], "fell_back": bool(rep["fell_back"]),
                            "history": [float(v) for v in hn]}
            # The same network solve with the inner basis in FP32, against the
            # mixed solve with that basis (the fastest mixed form).
            op.set_inner_basis(ls.LS_INNER_BASIS_F32)
            tn32, (xn32, hn32, rep32, coden32) = timed(
                lambda: op.fgmres_nn(net, b, flags=ls.LS_NN_GUESS | ls.LS_NN_PRECOND, max_outer=20,
                                     inner_iter=args.max_iter, tol=1e-8))
            op.set_inner_basis(ls.LS_INNER_BASIS_F64)
            nn["nn_fp32_basis"] = {"s": tn32, "converged": coden32 == 0, "true_residual": rep32["rel_residual"],
                                   "rel_err_vs_fp64": err_vs_fp64(xn32),
                                   "fp32_applies_and_fp64_products": rep32["n_matvec"],
                                   "network_applies": rep32["n_precond"], "history": [float(v) for v in hn32],
                                   "speedup_vs_fp64": t64 / tn32, "speedup_vs_mixed_fp32_basis": tm32 / tn32}
            nn["speedup_nn_vs_fp64"] = t64 / nn["nn"]["s"]
            nn["speedup_nn_vs_mixed"] = tm / nn["nn"]["s"]
            solve["nn_fgmres"] = nn
            net.close()
    # The reference's default (adaptive) tree at its published configuration.
    if solve is not None and not args.no_adaptive:
        solve["adaptive_readme"] = adaptive_leg(ls, local, timed, args.max_iter)
    # Many incidence directions on the scatterer (64 plane waves): the
    # batched mixed-precision solve against the same solves one at a time.
    batch = None
    if not args.no_solve and not args.no_batch:
        op.enable_f32()
        thetas = 2 * np.pi * np.arange(args.angles) / args.angles
        B = op.rhs_angles(thetas)
        # FP32 block applies with resident inputs: 64 right-hand sides on the
        # tensor cores against 8 on the CUDA-core block kernels.
        ms_tc = op.time_block_apply(64, warmup=3, iters=10)
        ms_cc = op.time_block_apply(8, warmup=3, iters=10)
        # The tensor-core apply's roofline: 12 TF32 MMAs (N <= 64) per stage,
        # each costing a fixed issue time below N = 128 (measured).
        tc_stages = op.tc_stages()
        mma_cycles = ls.measure_mma_issue(local, 48)
        sm_count = torch.cuda.get_device_properties(local).multi_processor_count
        clk_now = clk.summary()
        sm_mhz = clk_now.get("sm_mhz") or clk_now.get("sm_max_mhz") or 2070.0
        tc_floor_ms = tc_stages * 12 * mma_cycles / sm_count / (sm_mhz * 1e6) * 1e3
        op.set_batch_width(8)
        op.gmres_mixed_batched(B[:, :8], max_outer=20, inner_iter=100, tol=1e-8)  # warm-up: workspace
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Xb8, nmvb8, rrb8, codeb8 = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
        tb8 = time.perf_counter() - t0
        op.set_batch_width(64)
        op.gmres_mixed_batched(B[:, :8], max_outer=20, inner_iter=100, tol=1e-8)  # warm-up: workspace
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Xb, nmvb, rrb, codeb = op.gmres_mixed_batched(B, max_outer=20, inner_iter=100, tol=1e-8)
        tb = time.perf_counter() - t0
        t0 = time.perf_counter()
        rr_seq = []
        for j in range(B.shape[1]):
            _, _, _, rrj, _ = op.gmres_mixed(B[:, j], max_outer=20, inner_iter=args.max_iter, tol=1e-8)
            rr_seq.append(rrj)
        ts = time.perf_counter() - t0
        batch = {"nrhs": int(B.shape[1]), "directions": "2 pi m / %d" % args.angles, "tol": 1e-8,
                 "batched_s": tb, "batched_per_rhs_ms": tb / B.shape[1] * 1e3, "batched_block_applies_and_fp64_products": nmvb,
                 "batched_max_true_residual": float(np.max(rrb)), "batched_converged": codeb == 0,
                 "sequential_mixed_s": ts, "sequential_max_true_residual": float(np.max(rr_seq)),
                 "speedup_batched_vs_sequential": ts / tb, "block_width": 64,
                 "block_apply": {"tensor_core_64_ms": ms_tc, "tensor_core_per_rhs_us": ms_tc / 64 * 1e3,
                                 "cuda_core_8_ms": ms_cc, "cuda_core_per_rhs_us": ms_cc / 8 * 1e3,
                                 "speedup_per_rhs": (ms_cc / 8) / (ms_tc / 64),
                                 "issue_roofline": {"bound": "tensor-core MMA issue", "stages": tc_stages,
                                                    "mmas": 12 * tc_stages, "cycles_per_mma": mma_cycles,
                                                    "sm_mhz": sm_mhz, "floor_ms": tc_floor_ms,
                                                    "frac": tc_floor_ms / ms_tc}},
                 "width8": {"s": tb8, "block_applies_and_fp64_products": nmvb8,
                            "max_true_residual": float(np.max(rrb8)), "converged": codeb8 == 0,
                            "max_rel_diff_vs_width64": float(max(np.linalg.norm(Xb[:, j] - Xb8[:, j]) /
                                                                 np.linalg.norm(Xb8[:, j]) for j in range(B.shape[1])))}}
    # The many-scatterer workload: 32 seeded scatterers of uneven size (levels 4-6,
    # kappa U[10, 60], 1-4 bumps) x 64 directions, host assembly of the next
    # scatterer overlapped with the GPU solve of the current one.
    many = None
    if not args.no_solve and not args.no_batch and args.scatterers > 0:
        from lippmann_schwinger_solver_gb300 import scatterers as scat
        specs = scat.scatterer_specs(args.scatterers, SEED)
        recs, many, _ = scat.solve_many(specs, args.angles, 1e-8, 10, device=local)
        many["levels"] = {str(lv): sum(1 for r in recs if r["level"] == lv) for lv in (4, 5, 6)}
        many["host_stages_s"] = {k: round(sum(r["host_stages_s"][k] for r in recs), 2)
                                 for k in recs[0]["host_stages_s"]}
        # The same workload with the precomputation quadratures on the GPU
        # (not bit-exact with the oracle; every direction still meets the
        # FP64 true residual of its operator).
        recs_g, many_g, _ = scat.solve_many(specs, args.angles, 1e-8, 10, device=local, precompute_on_gpu=1)
        many_g["host_stages_s"] = {k: round(sum(r["host_stages_s"][k] for r in recs_g), 2)
                                   for k in recs_g[0]["host_stages_s"]}
        many["gpu_precompute"] = many_g
        # And with the far-field table and NCA on the GPU as well.
        recs_f, many_f, _ = scat.solve_many(specs, args.angles, 1e-8, 10, device=local, precompute_on_gpu=1,
                                            far_on_gpu=3)
        many_f["host_stages_s"] = {k: round(sum(r["host_stages_s"][k] for r in recs_f), 2)
                                   for k in recs_f[0]["host_stages_s"]}
        many["gpu_precompute_and_far"] = many_f
        # The same, two scatterers assembled and two solved at a time.
        _, many_w, _ = scat.solve_many(specs, args.angles, 1e-8, 10, device=local, precompute_on_gpu=1,
                                       far_on_gpu=3, workers=2)
        many["gpu_precompute_and_far_2_workers"] = many_w
    far_gpu = None
    if rank == 0 and not args.no_gpu_assembly:
        far_gpu = gpu_assembly_leg(ls, cfg, x, y_main, op.skeleton_dump(), local)
    peak, peak_kind = load_peaks()
    achieved = info["m2l_bytes"] / (ms_m2l * 1e-3) / 1e9
    traffic = traffic_per_launch(args.f64_kernels)
    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, parity = oracle_leg(ls, cfg, y_main, op.skeleton_dump(), budget_s=args.cpu_budget)
        if not (parity["rel_l2_vs_oracle"] <= parity["tolerance"] and parity["skeletons_equal"]):
            raise SystemExit("bench: GPU matvec differs from the oracle at the benchmark size: " + json.dumps(parity))
    # Measured FP64 FMA peak: the roof of the native FP64 kernels.
    fp64_peak = ls.measure_fma_peak(local, "fp64")
    fp32_peak = ls.measure_fma_peak(local, "fp32")
    phases = op.time_matvec_phases(warmup=3, iters=max(5, args.steps))
    d_bases = cfg.degreeOfBases
    n_bases = d_bases * (d_bases + 1) // 2  # Chebyshev T_a(x) T_b(y) with a + b < degreeOfBases
    side = int(round(info["n_leaves"] ** 0.5))
    pairs = (3 * side - 2) ** 2  # (leaf, colleague) pairs of a uniform side x side leaf grid
    # FP64 flops of the factored native near field: c = Q+ x per leaf (real x
    # complex) and Vt_q c per (leaf, colleague) and row (complex).
    near_f64_flops = 4 * info["n_leaves"] * n_bases * info["rank"] + 8 * pairs * info["rank"] * n_bases
    line = {
        "metric": METRIC, "value": value, "unit": "matvec/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128 (double-float: FP32 hi/lo pairs, 48-bit significand)" if df_kernels else "c128 (f64)",
        "data": "synthetic",
        "config": {"workload": "uniform level %d, N=%d, kappa=40, 3 seeded bumps (seed %d), NCA tol 1e-10"
                   % (args.level, n, SEED), "parallelism": "replicas" if world > 1 else "single GPU",
                   "f64_kernels": args.f64_kernels,
                   "l2": "inputs larger than L2: %.0f MB of operator blocks streamed per matvec"
                         % (info["far_entries"] * 16 / 1e6)},
        "e2e": {"value": world / e2e_s, "unit": "matvec/s", "h2d_bytes_per_step": 16 * n,
                "d2h_bytes_per_step": 16 * n},
        "gpu_launches": info["n_kernels_per_matvec"] * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind, "kernel": ("gemv_df_kernel<1> (M2L)" if df_kernels else "gemv_tiles_kernel<double2, 1> (M2L)"),
                     "kernel_ms": ms_m2l, "kernel_gflops_fp64": info["m2l_flops"] / (ms_m2l * 1e-3) / 1e9,
                     "fp64_pipe": {"peak_tflops": fp64_peak, "peak_source": "measured (ls_measure_fma_peak, DFMA chains)",
                                   "fp32_peak_tflops": fp32_peak,
                                   "m2l_tflops": info["m2l_flops"] / (ms_m2l * 1e-3) / 1e12,
                                   "m2l_frac": info["m2l_flops"] / (ms_m2l * 1e-3) / 1e12 / fp64_peak,
                                   "near_field_ms": phases["near"], "near_field_fp64_flops": near_f64_flops,
                                   "near_field_frac": (near_f64_flops / (phases["near"] * 1e-3) / 1e12 / fp64_peak
                                                       if not df_kernels else None),
                                   "matvec_fp64_flops": 8 * info["far_entries"] + near_f64_flops,
                                   "matvec_frac": ((8 * info["far_entries"] + near_f64_flops) / (ms * 1e-3) / 1e12
                                                   / fp64_peak if not df_kernels else None)}},
        "phases_ms": phases,
        "parity": parity,
        "matvec": {"bytes": info["matvec_bytes"], "flops_fp64": info["matvec_flops"],
                   "achieved_gbs": info["matvec_bytes"] / (ms * 1e-3) / 1e9,
                   "achieved_fp64_tflops": info["matvec_flops"] / (ms * 1e-3) / 1e12,
                   "assemble_s": info["assemble_seconds"], "device_bytes": info["device_bytes"],
                   "assemble_stages_s": dict(zip(("geometry", "precompute", "lists", "nca", "checks", "pack"),
                                                 (round(t, 3) for t in info["assemble_stage_seconds"]))),
                   "far_entries": info["far_entries"], "max_rank": info["max_rank"],
                   "far_on_gpu": far_gpu},
        "clocks": clk.summary(),
        "other_f64_kernels": alt,
        "solve": solve,
        "batched_solve": batch,
        "many_scatterers": many,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    op.close()
    if dist:
        dist.destroy_process_group()


def run_fno_forward(args):
    """Times `args.fno_forward` batch-1 forward passes of the trained
    network (the preconditioner's unit of work) with CUDA events; one JSON
    line. Also the command that the network's ncu launch lists profile."""
    import torch

    import lippmann_schwinger_solver_gb300 as ls
    net = ls.FNO.load(FNO_WEIGHTS)
    G = net.shape["grid"]
    st = torch.cuda.current_stream().cuda_stream
    x = torch.randn(1, G * G, ls.FNO_IN_CHANNELS, device="cuda")
    o = torch.empty(1, G * G, ls.FNO_OUT_CHANNELS, device="cuda")
    for _ in range(2):
        net.forward_device(1, x.data_ptr(), o.data_ptr(), stream=st)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.fno_forward):
        net.forward_device(1, x.data_ptr(), o.data_ptr(), stream=st)
    b.record()
    torch.cuda.synchronize()
    print(json.dumps({"metric": "spectral neural operator forward, batch 1", "unit": "ms",
                      "value": a.elapsed_time(b) / args.fno_forward, "passes": args.fno_forward,
                      "grid": G, "params": net.n_params}), flush=True)
    net.close()


def run_block_apply(args):
    """Times `--steps` FP32 block applies of `args.block_apply` right-hand
    sides (64: tensor cores, 8: CUDA cores) on the workload operator at
    `--level`, inputs resident; one JSON line. Also the command that the
    tensor-core kernel's ncu captures profile."""
    import lippmann_schwinger_solver_gb300 as ls
    op = ls.Operator(workload_config(ls, args.level), device=0)
    op.enable_f32()
    ms = op.time_block_apply(args.block_apply, warmup=max(3, args.warmup), iters=max(1, args.steps))
    print(json.dumps({"metric": "FP32 block apply", "unit": "ms", "value": ms, "width": args.block_apply,
                      "per_rhs_us": ms / args.block_apply * 1e3, "N": op.N, "level": args.level,
                      "tensor_core_stages": op.tc_stages()}), flush=True)
    op.close()


def run_profile_solve(args):
    """One FP64 GMRES and one mixed-precision solve to 1e-8 on the workload
    operator at `--level`, after an untimed pair, inside a CUDA profiler range
    (ncu --profile-from-start off captures just them); one JSON line."""
    import torch

    import lippmann_schwinger_solver_gb300 as ls
    op = ls.Operator(workload_config(ls, args.level), device=0)
    op.enable_f32()
    b = op.rhs()
    op.gmres(b, max_iter=args.max_iter, tol=1e-8)
    op.gmres_mixed(b, max_outer=20, inner_iter=args.max_iter, tol=1e-8)
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    _, _, it, rr, _ = op.gmres(b, max_iter=args.max_iter, tol=1e-8)
    t1 = time.perf_counter()
    _, _, nmv, rrm, _ = op.gmres_mixed(b, max_outer=20, inner_iter=args.max_iter, tol=1e-8)
    t2 = time.perf_counter()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"metric": "solve to 1e-8 inside a profiler range", "fp64_gmres_s": t1 - t0, "fp64_iters": it,
                      "fp64_true_residual": rr, "mixed_s": t2 - t1, "mixed_matvecs": nmv, "mixed_true_residual": rrm,
                      "N": op.N, "level": args.level}), flush=True)
    op.close()


def run_adaptive_matvecs(args):
    """Times `args.adaptive_matvecs` FP64 matvecs of the adaptive operator of
    the reference's README run with CUDA events (device-resident x); one
    JSON line. Also the command that its launch lists profile."""
    import lippmann_schwinger_solver_gb300 as ls
    op = ls.Operator(readme_adaptive_config(ls), device=0)
    ms = _device_matvec_ms(op, args.adaptive_matvecs, max(3, args.warmup))
    print(json.dumps({"metric": "FP64 matvec, adaptive README tree", "unit": "matvec/s", "value": 1e3 / ms,
                      "ms": ms, "N": op.N, "launches_per_matvec": op.info["n_kernels_per_matvec"],
                      "matvec_bytes": op.info["matvec_bytes"]}), flush=True)
    op.close()


def run_far_assembly(args):
    """Only the far-field-on-GPU assemblies of the workload against the host
    assembly (one JSON line)."""
    import lippmann_schwinger_solver_gb300 as ls

    ls.build()
    cfg = workload_config(ls, args.level)
    op = ls.Operator(cfg, device=0)
    x = input_vector(op.N)
    y = op.matvec(x)
    ih = op.info
    line = {"workload": "uniform level %d, N=%d, kappa=40, 3 seeded bumps, NCA tol 1e-10" % (args.level, op.N),
            "host_assemble_s": ih["assemble_seconds"],
            "host_stages_s": dict(zip(("geometry", "precompute", "lists", "nca", "checks", "pack"),
                                      (round(t, 3) for t in ih["assemble_stage_seconds"]))),
            "far_on_gpu": gpu_assembly_leg(ls, cfg, x, y, op.skeleton_dump(), 0)}
    print(json.dumps(line), flush=True)
    op.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the many-direction batched solve")
    ap.add_argument("--no-nn", action="store_true", help="skip the learned-preconditioner solve")
    ap.add_argument("--no-adaptive", action="store_true", help="skip the adaptive-tree operator at the README run")
    ap.add_argument("--no-gpu-assembly", action="store_true",
                    help="skip the operators assembled with their far field on the GPU")
    ap.add_argument("--far-assembly", action="store_true",
                    help="only compare the GPU far-field assemblies with the host one at this level")
    ap.add_argument("--angles", type=int, default=64, help="incidence directions of the batched solve")
    ap.add_argument("--scatterers", type=int, default=32,
                    help="scatterers of the many-scatterer batched workload (0 skips it)")
    ap.add_argument("--max-iter", type=int, default=400)
    ap.add_argument("--f64-kernels", default="native", choices=["native", "double-float"],
                    help="kernels behind the FP64 operator: FP64 arithmetic, or FP32 hi/lo pairs with "
                         "error-free transformations (same operator)")
    ap.add_argument("--precision", default="f64", choices=["f64", "f32"],
                    help="operator precision of the timed loop (f32: profiling run of the FP32 operator)")
    ap.add_argument("--fno-forward", type=int, default=0,
                    help="only time this many batch-1 forward passes of the trained network")
    ap.add_argument("--block-apply", type=int, default=0,
                    help="only time FP32 block applies of this many right-hand sides (64 or 8)")
    ap.add_argument("--adaptive-matvecs", type=int, default=0,
                    help="only time this many FP64 matvecs of the adaptive README-run operator")
    ap.add_argument("--profile-solve", action="store_true",
                    help="only run one FP64 and one mixed solve inside a CUDA profiler range")
    args = ap.parse_args()
    if args.fno_forward > 0:
        run_fno_forward(args)
    elif args.block_apply > 0:
        run_block_apply(args)
    elif args.profile_solve:
        run_profile_solve(args)
    elif args.adaptive_matvecs > 0:
        run_adaptive_matvecs(args)
    elif args.far_assembly:
        run_far_assembly(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
