"""Tile-shape autotuner for the gather-GEMV phases.

The assembler packs each phase's blocks into warp tiles of at most `rows`
rows (1, 2, 4 or 8) and aims the tile count at `warps` warps per SM
(csrc/assemble.cpp, `finalize`). This tool times candidate settings on the
GPU for one workload, phase kind by phase kind (upward M2M, M2L, downward
L2L; coordinate descent from the defaults 8 rows, 48 warps), and reports the
best. Each candidate is a full assembly with LS_TILE_<KIND>="rows,warps" in
the environment, then CUDA-event timings of the matvec with the native FP64,
double-float and FP32 kernels (the tiles are shared by all three); the
objective is the sum of the three times.

    python -m lippmann_schwinger_solver_gb300.autotune --level 6

Apply a result by exporting the printed LS_TILE_* variables before creating
operators.
"""
import argparse
import itertools
import json
import os
import time

from . import LS_F64_DOUBLE_FLOAT, LS_F64_NATIVE, LS_PREC_F32, LS_PREC_F64, Config, Operator, seeded_bumps

KINDS = ("M2L", "UP", "DOWN")
DEFAULT = (8, 48)


def workload(level, kappa=40.0, tol_pow=10, seed=20261203):
    return Config(nCones_LFR=16, nChebNodes=6, yes2DFMM=1, TOL_POW=tol_pow, degreeOfBases=6, nLevelsUniform=level,
                  Qchoice=6, findPhi=1, reference_rounding=1, L=1.0, kappa=kappa, bumps=seeded_bumps(seed))


def time_setting(cfg, setting, device=0, iters=20, repeats=3):
    """{kind: (rows, warps)} -> matvec ms with native, double-float, FP32."""
    saved = {k: os.environ.get("LS_TILE_" + k) for k in KINDS}
    try:
        for k in KINDS:
            r, w = setting.get(k, DEFAULT)
            os.environ["LS_TILE_" + k] = f"{r},{w}"
        op = Operator(cfg, device=device)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop("LS_TILE_" + k, None)
            else:
                os.environ["LS_TILE_" + k] = v
    try:
        out = {}
        op.set_f64_kernels(LS_F64_NATIVE)
        out["native"] = min(op.time_matvec(3, iters, LS_PREC_F64)[0] for _ in range(repeats))
        op.set_f64_kernels(LS_F64_DOUBLE_FLOAT)
        out["double_float"] = min(op.time_matvec(3, iters, LS_PREC_F64)[0] for _ in range(repeats))
        op.set_f64_kernels(LS_F64_NATIVE)
        op.enable_f32()
        out["fp32"] = min(op.time_matvec(3, iters, LS_PREC_F32)[0] for _ in range(repeats))
        out["sum"] = out["native"] + out["double_float"] + out["fp32"]
        return out
    finally:
        op.close()


def tune(cfg, rows=(2, 4, 8), warps=(24, 48, 96), device=0, log=print):
    best = {k: DEFAULT for k in KINDS}
    t0 = time.time()
    base = time_setting(cfg, best, device)
    log(json.dumps({"setting": "default", **{k: round(v, 4) for k, v in base.items()}}))
    best_t = base
    trials = []
    for kind in KINDS:
        for r, w in itertools.product(rows, warps):
            if (r, w) == best[kind]:
                continue
            cand = dict(best)
            cand[kind] = (r, w)
            t = time_setting(cfg, cand, device)
            trials.append({"kind": kind, "rows": r, "warps": w, **{k: round(v, 4) for k, v in t.items()}})
            log(json.dumps(trials[-1]))
            if t["sum"] < best_t["sum"]:
                best, best_t = cand, t
    return {"default_ms": base, "tuned_ms": best_t, "tuned": {k: list(v) for k, v in best.items()},
            "env": {f"LS_TILE_{k}": f"{v[0]},{v[1]}" for k, v in best.items()},
            "gain": base["sum"] / best_t["sum"], "trials": len(trials) + 1, "seconds": round(time.time() - t0, 1)}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--level", type=int, default=6)
    ap.add_argument("--kappa", type=float, default=40.0)
    a = ap.parse_args(argv)
    res = tune(workload(a.level, a.kappa))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
