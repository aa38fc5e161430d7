"""The assembler's fast ACA building blocks equal their plain forms bit for bit.

csrc/assemble.cpp ranks ACA pivots with std::abs only for entries near the
largest squared magnitude, and writes the norm estimate's inner products and
the rank-1 updates in real arithmetic. tests/cpp/assembler_arith_check.cpp
compiles against that source with the library's host flags and compares all
three with a full std::abs scan and with std::complex arithmetic on 200,000
adversarial vectors: equal magnitudes at many phases, one-ulp differences,
signed zeros, values near underflow, random used-masks."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fast_aca_blocks_match_plain_forms(tmp_path):
    exe = str(tmp_path / "assembler_arith_check")
    src = os.path.join(ROOT, "tests", "cpp", "assembler_arith_check.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"),
                    src, "-o", exe], check=True, capture_output=True, timeout=600)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "pivot mismatches 0, inner-product mismatches 0, update mismatches 0" in out.stdout
