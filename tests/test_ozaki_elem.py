"""The Ozaki operand passes' element-wise arithmetic (momms_gb300/csrc/
ozaki_elem.cuh), compiled for the host, against exact rational arithmetic:

* exponent_of_max: the smallest e with |v| < 2^e (0 for zero, INT32_MAX for
  NaN / infinity);
* offset_digits<NS>: Y = round_half_up(|v| 2^(8 NS - e)) + H, H the offset
  that centres the lower digits (all zero for e == INT32_MAX);
* magnitude: |v| 2^-e as bf16 rounded toward zero (0 below bf16's normal
  range) and ceil(|v| 2^(40 - e)); the 0/1 indicator form.

Cases: normals over the whole exponent range, subnormals, exact halves at
the rounding position and their neighbours, zero, NaN / infinity rows, row
exponents from the element's own up to 60 above it, 1..15 digits.
"""
import math
import os
import random
import struct
import subprocess
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_ozaki_elem.cpp")
CSRC = os.path.join(ROOT, "momms_gb300", "csrc")
INT32_MAX = 2**31 - 1


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("elem") / "ozaki_elem")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-Wno-unknown-pragmas", "-I", CSRC,
                    SRC, "-o", out], check=True, capture_output=True, text=True)
    return out


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _run(exe, lines):
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return r.stdout.split("\n")


def _exp(v):
    if not math.isfinite(v):
        return INT32_MAX
    if v == 0:
        return 0
    return math.frexp(v)[1]


def _values(rng, n):
    vals = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 2.2250738585072009e-308, 1.0, -1.0,
            0.5, 1.7976931348623157e308, float("inf"), float("-inf"), float("nan")]
    for _ in range(n):
        kind = rng.random()
        if kind < 0.6:
            v = rng.uniform(0.5, 1.0) * 2.0 ** rng.randint(-1070, 1020)
        elif kind < 0.8:
            v = struct.unpack("<d", struct.pack("<Q", rng.randint(1, 2**52 - 1)))[0]  # subnormal
        else:
            v = rng.uniform(-1, 1)
        vals.append(v if rng.random() < 0.5 else -v)
    return vals


def test_exponent_of_max(exe):
    rng = random.Random(1)
    vals = _values(rng, 3000)
    out = _run(exe, [f"0 {_bits(v)}" for v in vals])
    for v, o in zip(vals, out):
        assert int(o) == _exp(abs(v)), v


def _offset(ns):
    return sum(128 << (8 * pos) for pos in range(ns - 1))


def _digits_case(v, e, ns):
    if e == INT32_MAX or v == 0:
        return _offset(ns)
    s = abs(Fraction(v)) * Fraction(2) ** (8 * ns - e)
    x = math.floor(s + Fraction(1, 2))  # halves round up
    return x + _offset(ns)


def test_offset_digits(exe):
    rng = random.Random(2)
    cases = []
    for v in _values(rng, 1500):
        e0 = _exp(abs(v))
        for ns in (1, 2, 3, 7, 8, 9, 13, 15):
            e = e0 if e0 == INT32_MAX else e0 + rng.choice([0, 0, 1, 3, 17, 60])
            cases.append((v, e, ns))
    # exact halves at the last digit and their neighbours: |v| 2^(8 ns - e) = q + 1/2
    for _ in range(600):
        ns = rng.choice([1, 2, 5, 7, 8, 12, 15])
        e = rng.randint(-900, 900)
        q = rng.randint(1, 2 ** min(8 * ns, 50) - 2)
        for num in (2 * q + 1, 2 * q):
            v = float(Fraction(num, 2) * Fraction(2) ** (e - 8 * ns))
            if v != 0 and math.isfinite(v) and abs(v) < 2.0 ** e:
                cases.append((v, e, ns))
                cases.append((math.nextafter(v, 0.0), e, ns))
                cases.append((math.nextafter(v, math.inf), e, ns))
    # the passes only use row exponents with |v| < 2^e
    cases = [c for c in cases if c[1] == INT32_MAX or abs(Fraction(c[0])) < Fraction(2) ** c[1]]
    out = _run(exe, [f"1 {_bits(v)} {e} {ns}" for v, e, ns in cases])
    for (v, e, ns), o in zip(cases, out):
        hi, lo = (int(t) for t in o.split())
        assert (hi << 64) | lo == _digits_case(v, e, ns), (v, e, ns)


def _magnitude_case(v, e, indicator):
    if v == 0 or e == INT32_MAX or not math.isfinite(v):
        return 0, 0
    if indicator:
        return 0x3F80, 0
    s = abs(Fraction(v)) * Fraction(2) ** (-e)
    fix = math.ceil(s * 2**40)
    X = math.floor(math.log2(s))
    while Fraction(2) ** X > s:
        X -= 1
    while Fraction(2) ** (X + 1) <= s:
        X += 1
    if X + 127 < 1:
        bf = 0
    else:
        mant = math.floor(s / Fraction(2) ** X * 128) - 128  # 7 fraction bits, toward zero
        bf = ((X + 127) << 7) | mant
    return bf, fix


def test_magnitude_terms(exe):
    rng = random.Random(3)
    cases = []
    for v in _values(rng, 2500):
        e0 = _exp(abs(v))
        for _ in range(3):
            e = e0 if e0 == INT32_MAX else e0 + rng.choice([0, 0, 1, 5, 40, 60, 150])
            cases.append((v, e, 0))
        cases.append((v, e0, 1))
    out = _run(exe, [f"2 {_bits(v)} {e} {ind}" for v, e, ind in cases])
    for (v, e, ind), o in zip(cases, out):
        bf, fix = (int(t) for t in o.split())
        assert (bf, fix) == _magnitude_case(v, e, ind), (v, e, ind)
