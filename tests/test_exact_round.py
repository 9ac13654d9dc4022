"""The recombination's integer -> double rounding (momms_gb300/csrc/
exact_round.cuh), compiled for the host, against exact rational rounding.

The Ozaki path forms each entry of C as one exact integer R (the group sums
of the digit products, up to 148 bits) times a power of two and rounds it to
double once; this is that single rounding. Python's Fraction -> float
conversion is correctly rounded (nearest, ties to even, gradual underflow),
so every result must match it bit for bit: random magnitudes of 1..126 bits,
forced ties and near-ties at the rounding position, results in the
subnormal range and past the largest double, and the four-partial wide form.
"""
import os
import random
import struct
import subprocess
from fractions import Fraction

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_exact_round.cpp")
CSRC = os.path.join(ROOT, "momms_gb300", "csrc")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("round") / "exact_round")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I", CSRC, SRC, "-o", out],
                   check=True, capture_output=True, text=True)
    return out


def _exact_bits(R, scale):
    f = Fraction(R) * Fraction(2) ** scale
    try:
        x = float(f)
    except OverflowError:
        x = float("inf") if R > 0 else float("-inf")
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _split128(R):
    u = R & ((1 << 128) - 1)
    hi, lo = u >> 64, u & ((1 << 64) - 1)
    return hi - (1 << 64) if hi >= 1 << 63 else hi, lo


def _cases(seed, count):
    rng = random.Random(seed)
    lines, want = [], []
    for _ in range(count):
        nb = rng.randint(1, 126)
        R = rng.getrandbits(nb) | (1 << (nb - 1))
        if nb > 2 and rng.random() < 0.4:
            # a tie or near-tie at a random rounding position
            t = rng.randint(1, nb - 1)
            R = (R >> t) << t
            if rng.random() < 0.5:
                R |= 1 << (t - 1)
            if rng.random() < 0.3:
                R |= 1
        r = rng.random()
        if r < 0.25:
            e = rng.randint(-1080, -1015)  # around and below the smallest normal
        elif r < 0.35:
            e = rng.randint(1015, 1030)  # around the largest double
        else:
            e = rng.randint(-900, 900)
        scale = e - (nb - 1)
        if rng.random() < 0.5:
            R = -R
        hi, lo = _split128(R)
        lines.append(f"0 {hi} {lo} {scale}")
        want.append(_exact_bits(R, scale))
    for _ in range(count):
        P = [rng.randint(-(1 << 62), 1 << 62) for _ in range(4)]
        r = rng.random()
        if r < 0.3:
            P[3] = 0
        elif r < 0.6:
            P[3] = rng.randint(-(1 << 20), 1 << 20)
        R = P[0] + (P[1] << 32) + (P[2] << 64) + (P[3] << 96)
        scale = rng.randint(-1100, 900)
        lines.append(f"1 {P[0]} {P[1]} {P[2]} {P[3]} {scale}")
        want.append(_exact_bits(R, scale))
    for R in (0, 1, -1, (1 << 126) - 1, -((1 << 126) - 1), 1 << 53, (1 << 53) + 1, (1 << 54) + 2, (1 << 54) + 6):
        hi, lo = _split128(R)
        lines.append(f"0 {hi} {lo} 0")
        want.append(_exact_bits(R, 0))
    return lines, want


@pytest.mark.parametrize("seed", [1, 2])
def test_rounding_matches_exact(exe, seed):
    lines, want = _cases(seed, 6000)
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in r.stdout.split()]
    assert len(got) == len(want)
    bad = [(lines[i], got[i], want[i]) for i in range(len(want)) if got[i] != want[i]]
    assert not bad, bad[:5]
