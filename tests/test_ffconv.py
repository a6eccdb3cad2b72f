"""The mixed path's float-float -> FP64 conversion (finetools.jl_gb300/csrc/
ffconv.h), compiled for the host and checked against exact rational
arithmetic on ~44,000 pairs (tests/ffconv_check.cpp):
  - ff_to_double_exact: the FP64 value nearest to h + l (ties to even) when
    l's bits reach at most 37 binades below h (else within one half unit plus
    the truncated part); zero / FP32-subnormal sums give signed zeros; inf
    and nan keep their class;
  - ff_to_double (the row gather's routine): the same bound (nearest FP64,
    ties to even) for every finite case, and equal to the exact routine on
    the special cases.
No GPU is involved.
"""
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _f(hexs):
    return struct.unpack(">f", bytes.fromhex(hexs))[0]


def _d(hexs):
    return struct.unpack(">d", bytes.fromhex(hexs))[0]


def _ulp(x):
    import math
    m, e = math.frexp(abs(x))
    return Fraction(2) ** (e - 53)


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_float_float_to_double(tmp_path):
    import math
    exe = str(tmp_path / "ffconv_check")
    cmd = ["g++", "-O1", "-std=c++17", "-ffp-contract=off", "-fno-fast-math",
           "-I", os.path.join(ROOT, "finetools.jl_gb300", "csrc"),
           os.path.join(ROOT, "tests", "ffconv_check.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout.split("\n")
    n_checked = 0
    for line in out:
        if not line.strip():
            continue
        hb, lb, eb, fb = line.split()
        h, l, ex, fa = _f(hb), _f(lb), _d(eb), _d(fb)
        if math.isnan(h) or math.isnan(l):
            assert math.isnan(ex) and math.isnan(fa)
            continue
        if math.isinf(h) or math.isinf(l):
            assert ex == h + l and fa == ex
            continue
        exact = Fraction(h) + Fraction(l)
        if abs(exact) < Fraction(2) ** -126:      # FP32-subnormal sums: signed zero
            assert ex == 0.0 and fa == 0.0
            continue
        # exact routine: within half an ulp (plus the bits it truncates)
        err_ex = abs(Fraction(ex) - exact)
        assert err_ex <= _ulp(ex) / 2 + abs(exact) * Fraction(2) ** -60, line
        # gather routine: nearest, ties to even
        err_fa = abs(Fraction(fa) - exact)
        assert err_fa <= _ulp(fa) / 2 + abs(exact) * Fraction(2) ** -60, line
        if err_fa == _ulp(fa) / 2:
            assert struct.unpack(">Q", struct.pack(">d", fa))[0] % 2 == 0, line
        n_checked += 1
    assert n_checked > 40000
