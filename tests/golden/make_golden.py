"""Generates the golden vectors in this directory from the reference's own code.

The reference publishes no golden vectors and its inputs are unseeded, so the
fixtures are made here: seeded inputs are pushed through the reference's own
BLIS Haswell microkernels (ukernels/bli_gemm_haswell_asm_d6x8.c, compiled
unmodified into oracle/_ref by oracle/build.py) inside the Goto loop nest of
the oracle (src/exper/l3_packing.rs:58-66 blocking). Needs an x86-64 host with
AVX2/FMA and the reference checkout; run from the repository root:

    python tests/golden/make_golden.py

Files written:
  ukr_golden.npz   single microkernel calls (d6x8 and s6x16), several k,
                   beta in {0, 1, -0.7}, row- and general-stored C
  goto_golden.npz  whole C := beta*C + alpha*A*B problems through the Goto nest
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from tests import oracle_util as ou  # noqa: E402

SEED = 20260301

UKR_CASES = [  # (k, beta, row_stored)
    (0, 0.0, True), (1, 1.0, True), (3, -0.7, False), (4, 0.0, False), (13, 1.0, False),
    (13, -0.7, True), (192, 1.0, True), (192, 0.0, False),
]

GOTO_CASES = [  # (m, n, k, alpha, beta, c_row_major)
    (1, 1, 1, 1.0, 1.0, False),
    (6, 8, 4, 1.0, 0.0, False),
    (7, 9, 13, 1.0, 1.0, True),
    (13, 17, 193, 0.75, -0.5, False),
    (121, 9, 24, 1.0, 1.0, True),
    (13, 11, 385, 1.0, 1.0, False),
    (2, 3010, 5, 1.0, 1.0, False),
    (125, 10, 1, -1.0, 0.25, True),
]


def aligned(x):
    buf = np.empty(x.size + 64, dtype=x.dtype)
    off = (-buf.ctypes.data % 64) // x.itemsize
    out = buf[off:off + x.size]
    out[:] = x.ravel()
    return out


def main():
    ref = ou.load_ref()
    if ref is None:
        raise SystemExit("needs x86-64 and the reference checkout (oracle/_ref)")
    rng = np.random.default_rng(SEED)
    ukr = {}
    for dt, tag, mr, nr, sym in ((np.float64, "d", 6, 8, "bli_dgemm_haswell_asm_6x8"),
                                 (np.float32, "s", 6, 16, "bli_sgemm_haswell_asm_6x16")):
        f = getattr(ref, sym)
        for ci, (k, beta, row_stored) in enumerate(UKR_CASES):
            a = aligned(rng.uniform(-1, 1, k * mr + 2 * mr).astype(dt))
            b = aligned(rng.uniform(-1, 1, k * nr + 2 * nr).astype(dt))
            rs, cs = (nr, 1) if row_stored else (1, 2 * mr)
            c0 = rng.uniform(-1, 1, 4 * mr * nr).astype(dt)
            c = c0.copy()
            al = np.array([0.9], dt)
            be = np.array([beta], dt)
            f(ctypes.c_int64(k), ou.ptr(al), ou.ptr(a), ou.ptr(b), ou.ptr(be), ou.ptr(c), ctypes.c_int64(rs),
              ctypes.c_int64(cs), None, None)
            key = f"{tag}{ci}"
            ukr[key + "_a"], ukr[key + "_b"], ukr[key + "_c0"], ukr[key + "_c"] = a, b, c0, c
            ukr[key + "_meta"] = np.array([k, rs, cs], np.int64)
            ukr[key + "_ab"] = np.array([0.9, beta], np.float64)
    np.savez_compressed(os.path.join(HERE, "ukr_golden.npz"), **ukr)

    goto = {}
    for dt, tag, sym in ((np.float64, "d", "bli_dgemm_haswell_asm_6x8"),
                         (np.float32, "s", "bli_sgemm_haswell_asm_6x16")):
        kern = ctypes.cast(getattr(ref, sym), ctypes.c_void_p)
        for ci, (m, n, k, alpha, beta, c_rm) in enumerate(GOTO_CASES):
            A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
            B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
            C0 = rng.uniform(-1, 1, (m, n)).astype(dt)
            C0 = np.ascontiguousarray(C0) if c_rm else np.asfortranarray(C0)
            C = C0.copy(order="A")
            ou.goto_gemm(A, B, C, alpha, beta, threads=4, ukr=kern)
            key = f"{tag}{ci}"
            goto[key + "_A"], goto[key + "_B"], goto[key + "_C0"], goto[key + "_C"] = A, B, C0, C
            goto[key + "_meta"] = np.array([m, n, k, int(c_rm)], np.int64)
            goto[key + "_ab"] = np.array([alpha, beta], np.float64)
    np.savez_compressed(os.path.join(HERE, "goto_golden.npz"), **goto)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
