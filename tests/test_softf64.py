"""The reference-order path's integer-unit FP64 addition (finetools.jl_gb300/
csrc/softf64.cuh, sf_add), compiled for the host and compared bit for bit
with the host's IEEE binary64 addition (tests/softf64_check.cpp) on 14
million operand pairs: uniform bit patterns (zeros, subnormals, infinities,
NaNs), exponent differences 0..70 with random signs, near-cancellations,
exact ties to even, sums at both ends of the normal range, signed zeros.
The device build of the same routine is compared with the FP64 unit's
__dadd_rn in tests/test_gpu_parity.py (fegpu_selftest_soft_add).
No GPU is involved.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_soft_add_matches_ieee_addition(tmp_path):
    exe = str(tmp_path / "softf64_check")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
           "-I", os.path.join(ROOT, "finetools.jl_gb300", "csrc"),
           os.path.join(ROOT, "tests", "softf64_check.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:]
    assert "14252004 sums, 0 mismatches" in r.stdout
