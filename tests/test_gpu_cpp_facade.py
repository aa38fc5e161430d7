"""The C++ facade (include/ls_dafmm.hpp) driven like the reference's main:
DFMM + classGMRES + RestartedGMRES through the C ABI, on the GPU."""
import json
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_reference_style_cpp_driver(ls):
    exe = os.path.join(os.path.dirname(ls.LIB_PATH), "gmres_driver")
    out = subprocess.run([exe, "4", "10", "8", "0"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["N"] == 9216
    assert r["estimate"] <= 1e-10
    assert r["residual"] <= 2e-10
    assert r["restarted_vs_tol"] <= 1e-6
    assert r["batched_max_residual"] <= 1.5e-8
    assert r["batched_applies"] > 0
    assert r["double_float_vs_native"] <= 2e-11
