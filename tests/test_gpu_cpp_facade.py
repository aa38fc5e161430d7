"""The C++ facade (include/ls_dafmm.hpp) driven like the reference's main:
DFMM + classGMRES + RestartedGMRES through the C ABI, on the GPU."""
import json
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_reference_style_cpp_driver(ls, tmp_path):
    pkg = os.path.dirname(ls.LIB_PATH)
    exe = os.path.join(pkg, "gmres_driver")
    result = tmp_path / "Phi_1_10"
    weights = os.path.join(pkg, "weights", "fno_k10_40.lsfno")
    args = [exe, "4", "10", "8", "0", str(result)] + ([weights] if os.path.exists(weights) else [])
    out = subprocess.run(args, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    lines = result.read_text().splitlines()
    assert len(lines) == r["N"] and lines[0].startswith("(") and lines[0].endswith(")")
    assert r["interpolation_error"] <= 1e-12
    if os.path.exists(weights):
        assert r["nn_residual"] <= 1.5e-8 and r["nn_network_applies"] >= 1
    assert r["N"] == 9216
    assert r["estimate"] <= 1e-10
    assert r["residual"] <= 2e-10
    assert r["restarted_vs_tol"] <= 1e-6
    assert r["batched_max_residual"] <= 1.5e-8
    assert r["batched_applies"] > 0
    assert r["double_float_vs_native"] <= 2e-11
