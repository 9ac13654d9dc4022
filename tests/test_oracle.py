"""The oracle pinned against the reference's own kernels (CPU only).

* The portable microkernels reproduce the reference's BLIS Haswell asm
  kernels bit for bit (golden vectors made by tests/golden/make_golden.py).
* The oracle's Goto loop nest reproduces the golden whole-problem results bit
  for bit.
* On x86-64 hosts with the reference checkout, the asm kernels are also run
  live against fresh seeded inputs.
* The double-double oracle and the Freivalds residual are checked on exact
  small-integer problems.
"""
import ctypes
import os
from fractions import Fraction

import numpy as np
import pytest

from tests import oracle_util as ou

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _aligned(x):
    buf = np.empty(x.size + 64, dtype=x.dtype)
    off = (-buf.ctypes.data % 64) // x.itemsize
    out = buf[off:off + x.size]
    out[:] = x.ravel()
    return out


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint8)


def _ukr_cases(data):
    tags = sorted({k.split("_")[0] for k in data.files})
    return tags


def test_ukr_golden_bitwise(oracle_lib):
    data = np.load(os.path.join(GOLDEN, "ukr_golden.npz"))
    n = 0
    for tag in _ukr_cases(data):
        k, rs, cs = (int(v) for v in data[tag + "_meta"])
        al, be = data[tag + "_ab"]
        dt = np.float64 if tag[0] == "d" else np.float32
        f = oracle_lib.oracle_ukr_d6x8 if tag[0] == "d" else oracle_lib.oracle_ukr_s6x16
        a = _aligned(data[tag + "_a"])
        b = _aligned(data[tag + "_b"])
        c = data[tag + "_c0"].copy()
        alv, bev = np.array([al], dt), np.array([be], dt)
        f(k, ou.ptr(alv), ou.ptr(a), ou.ptr(b), ou.ptr(bev), ou.ptr(c), rs, cs, None, None)
        assert np.array_equal(_bits(c), _bits(data[tag + "_c"])), tag
        n += 1
    assert n == 16


def test_goto_golden_bitwise(oracle_lib):
    data = np.load(os.path.join(GOLDEN, "goto_golden.npz"))
    tags = sorted({k.split("_")[0] for k in data.files})
    assert len(tags) == 16
    for tag in tags:
        A, B, C0 = data[tag + "_A"], data[tag + "_B"], data[tag + "_C0"]
        alpha, beta = (float(v) for v in data[tag + "_ab"])
        for threads in (1, 3):
            C = C0.copy(order="A")
            ou.goto_gemm(A, B, C, alpha, beta, threads=threads)
            assert np.array_equal(_bits(C), _bits(data[tag + "_C"])), (tag, threads)


def test_goto_k0_leaves_c(oracle_lib):
    A = np.zeros((5, 0), order="F")
    B = np.zeros((0, 4), order="F")
    C = np.asfortranarray(np.arange(20.0).reshape(5, 4))
    C0 = C.copy(order="F")
    ou.goto_gemm(A, B, C, 1.0, 0.0)
    assert np.array_equal(C, C0)


@pytest.mark.skipif(ou.load_ref() is None, reason="reference asm kernels need x86-64 + the reference checkout")
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_live_reference_kernels_match_port(dt):
    ref = ou.load_ref()
    sym = "bli_dgemm_haswell_asm_6x8" if dt == np.float64 else "bli_sgemm_haswell_asm_6x16"
    kern = ctypes.cast(getattr(ref, sym), ctypes.c_void_p)
    rng = np.random.default_rng(7)
    for (m, n, k) in [(1, 1, 1), (7, 9, 13), (130, 250, 400), (241, 19, 200)]:
        A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
        B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
        C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
        C1, C2 = C0.copy(order="F"), C0.copy(order="F")
        ou.goto_gemm(A, B, C1, 1.0, 1.0, threads=4, ukr=kern)
        ou.goto_gemm(A, B, C2, 1.0, 1.0, threads=4)
        assert np.array_equal(_bits(C1), _bits(C2))


def test_dd_oracle_exact_on_integers(oracle_lib):
    rng = np.random.default_rng(3)
    m, n, k = 5, 4, 9
    # entries with 30 significant bits: products exceed 2^53, so plain f64 rounds
    A = np.asfortranarray(rng.integers(-2**30, 2**30, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-2**30, 2**30, (k, n)).astype(np.float64))
    C0 = np.asfortranarray(rng.integers(-2**40, 2**40, (m, n)).astype(np.float64))
    out, mag = ou.dd_gemm(A, B, C0, alpha=1.0, beta=1.0)
    for i in range(m):
        for j in range(n):
            exact = Fraction(int(C0[i, j])) + sum(Fraction(int(A[i, p])) * int(B[p, j]) for p in range(k))
            assert out[i, j] == float(exact)
            assert mag[i, j] == pytest.approx(float(sum(abs(A[i, p] * B[p, j]) for p in range(k)) + abs(C0[i, j])))
    ii = np.array([0, 4, 2])
    jj = np.array([3, 0, 1])
    e_out, _ = ou.dd_gemm_entries(A, B, C0, ii, jj)
    assert np.array_equal(e_out, out[ii, jj])


def test_goto_within_bound_of_dd(oracle_lib):
    rng = np.random.default_rng(11)
    m, n, k = 67, 45, 500
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    C = C0.copy(order="F")
    ou.goto_gemm(A, B, C, 1.0, 1.0)
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.bound_ratio(C, ref, mag, k, 2.0**-53) <= 1.0
    # float32 at FP32 u
    A32, B32, C32 = (np.asfortranarray(x.astype(np.float32)) for x in (A, B, C0))
    C = C32.copy(order="F")
    ou.goto_gemm(A32, B32, C, 1.0, 1.0)
    ref, mag = ou.dd_gemm(A32, B32, C32)
    assert ou.bound_ratio(C, ref, mag, k, 2.0**-24) <= 1.0


def test_freivalds_residual(oracle_lib):
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.integers(-8, 8, (9, 7)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-8, 8, (7, 6)).astype(np.float64))
    C = np.asfortranarray(A @ B)
    w = rng.integers(-3, 4, 6).astype(np.float64)
    assert ou.freivalds(A, B, C, w) == 0.0
    C[2, 3] += 1.0
    assert ou.freivalds(A, B, C, w) > 0.0 or w[3] == 0.0
