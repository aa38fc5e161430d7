"""bench.py's JSON line: the keys and types the benchmark contract asks for.
The reference arm (the oracle port on the host cores) runs here on the CPU
at a small level; our arm runs on the GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args, timeout=900):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                         timeout=timeout, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def _common(r):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline"):
        assert k in r, k
    assert r["value"] > 0 and r["unit"] == "matvec/s" and r["higher_is_better"] is True
    assert r["warmup"] >= 3 and r["scaling"] in ("weak", "strong")
    assert "workload" in r["config"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in r["e2e"], k


def test_reference_arm_contract():
    r = _run(["--impl", "reference", "--level", "3", "--steps", "2", "--warmup", "3"])
    _common(r)
    assert r["impl"] == "reference" and "level 3" in r["config"]["workload"]
    assert r["cpu_baseline"]["kind"] in ("port", "reference") and r["cpu_baseline"]["cores"] >= 1
    assert r["e2e"]["h2d_bytes_per_step"] == 0


@pytest.mark.gpu
def test_our_arm_contract():
    r = _run(["--level", "4", "--steps", "5", "--warmup", "3", "--cpu-budget", "1", "--no-batch", "--no-nn"])
    _common(r)
    assert r["n_gpus"] == 1 and r["gpu_launches"] > 0
    rf = r["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in rf, k
    assert 0 < rf["frac"] < 1.5 and rf["unit"] == "GB/s"
    assert r["e2e"]["h2d_bytes_per_step"] == 16 * int(r["config"]["workload"].split("N=")[1].split(",")[0])
    assert "sm_mhz" in r["clocks"] and r["solve"]["fp64_converged"] and r["solve"]["mixed_converged"]
    # parity with the oracle on the benchmark input, and the CPU baseline's parts
    assert r["parity"]["skeletons_equal"] and r["parity"]["rel_l2_vs_oracle"] <= 1e-10
    cb = r["cpu_baseline"]
    assert cb["one_thread"]["cores"] == 1 and cb["cpu_model"] and cb["solve_s"]["workload_true_residual"] <= 1e-8
    fp = rf["fp64_pipe"]
    assert fp["peak_tflops"] > 0 and 0 < fp["m2l_frac"] < 1.5 and 0 < fp["near_field_frac"] < 1.5
    assert set(r["phases_ms"]) == {"total", "up", "m2l", "down", "near"}
    assert r["solve"]["mixed_rel_err_vs_fp64"] < 1e-6
    # the adaptive operator at the reference's published run reproduces its residuals
    ad = r["solve"]["adaptive_readme"]
    assert ad["N"] == 5328 and ad["fp64_converged"] and ad["mixed_converged"]
    for restarts in ("1", "2"):
        assert ad["restarted_gmres_m10"][restarts]["rel_diff"] <= 2e-5, ad["restarted_gmres_m10"]
