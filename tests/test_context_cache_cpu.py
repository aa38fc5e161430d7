"""The static scratch array's device address is cached per device and per
CUDA context (csrc/context_cache.h): looked up again when the context
changes, as after cudaDeviceReset, so the allocation-free matvec never uses
an address from a destroyed context. tests/cpp/context_cache_check.cpp
drives the cache with fake context IDs; no GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_context_cache_refetches_on_context_change(tmp_path):
    exe = str(tmp_path / "context_cache_check")
    src = os.path.join(ROOT, "tests", "cpp", "context_cache_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", src, "-o", exe], check=True, capture_output=True, timeout=300)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "context cache checks: 0 failed" in out.stdout
