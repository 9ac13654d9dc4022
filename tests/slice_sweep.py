"""Error and speed of emulated FP64 against the slice count, on the emulation
inputs a_ij = U[-0.5, 0.5] exp(phi N(0, 1)) (m = n = k = s):

  * s in {2048, 4096, 8192}, phi in {0.5, 2, 8};
  * fixed slice counts 3..9 and the automatic count at a 1e-14 target;
  * error: max over the checked entries of |C_ij - exact_ij| / (|A||B|)_ij,
    exact_ij from the double-double oracle (oracle/goto.c), on every entry at
    s = 2048 and on whole rows (512 at 4096, 128 at 8192, seeded) above;
  * speed: device-resident operands, one warm-up call, then three calls timed
    with CUDA events; effective FP64 TFLOP/s = 2 s^3 / time; plain DGEMM on
    the same inputs beside it.

    python -m tests.slice_sweep [--sizes 2048 4096 8192] > sweep.md

Prints one JSON line per cell and a markdown table at the end. It runs the
oracle, so it lives with the tests, not in the package.
"""
import argparse
import ctypes
import json
import sys

import numpy as np

import momms_gb300 as mg
from tests import oracle_util as ou

ROWS_CHECKED = {2048: None, 4096: 512, 8192: 128}


def _operands(s, phi, seed):
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (s, s)) * np.exp(phi * rng.standard_normal((s, s))))
    B = np.asfortranarray(rng.uniform(-0.5, 0.5, (s, s)) * np.exp(phi * rng.standard_normal((s, s))))
    return A, B


def _call(lib, torch, dA, dB, dC, s, precision, slices=0, target=0.0, reps=3):
    d = mg.GemmDesc()
    d.dtype, d.precision = mg.DTYPE_F64, precision
    d.m = d.n = d.k = s
    d.alpha, d.beta = 1.0, 0.0
    d.a = mg.Operand(dA.data_ptr(), 1, s, mg.MEM_DEVICE, 0)
    d.b = mg.Operand(dB.data_ptr(), 1, s, mg.MEM_DEVICE, 0)
    d.c = mg.Operand(dC.data_ptr(), 1, s, mg.MEM_DEVICE, 0)
    d.slices = slices
    d.target_rel_err = target
    st = torch.cuda.current_stream()
    sp = ctypes.c_void_p(st.cuda_stream)
    rc = lib.momms_gemm(ctypes.byref(d), sp)
    if rc not in (mg.OK, mg.ERR_TARGET_UNREACHABLE):
        mg.check(rc, lib)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        rc = lib.momms_gemm(ctypes.byref(d), sp)
        if rc not in (mg.OK, mg.ERR_TARGET_UNREACHABLE):
            mg.check(rc, lib)
    e1.record(st)
    e1.synchronize()
    info = mg.CallInfo()
    lib.momms_last_info(ctypes.byref(info))
    return rc, e0.elapsed_time(e1) / reps, info


def sweep(sizes, phis=(0.5, 2.0, 8.0), slice_range=range(3, 10), out=sys.stdout):
    import torch
    lib = mg.load_library()
    rows_out = []
    for s in sizes:
        for phi in phis:
            A, B = _operands(s, phi, seed=int(phi * 100) + s)
            nrows = ROWS_CHECKED.get(s)
            if nrows is None:
                rows = np.arange(s)
            else:
                rows = np.sort(np.random.default_rng(s + 1).choice(s, nrows, replace=False))
            ref, mag = ou.dd_gemm(np.asfortranarray(A[rows, :]), B, None, beta=0.0)
            dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()
            dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda().t()
            dC = torch.zeros((s, s), dtype=torch.float64, device="cuda").t()
            cells = [("plain", mg.PREC_PLAIN, 0, 0.0)] + [(f"{n}", mg.PREC_OZAKI, n, 0.0) for n in slice_range]
            cells.append(("auto 1e-14", mg.PREC_OZAKI, 0, 1e-14))
            for name, prec, ns, target in cells:
                reps = 1 if (prec == mg.PREC_PLAIN and s >= 4096) else 3
                rc, ms, info = _call(lib, torch, dA, dB, dC, s, prec, ns, target, reps)
                C = dC.t().cpu().numpy().T[rows, :]
                err = ou.rel_err(C, ref, mag)
                row = {"s": s, "phi": phi, "slices": name, "used": int(info.slices) if prec else 0, "ms": ms,
                       "tflops": 2.0 * s**3 / (ms * 1e-3) / 1e12, "err": err,
                       "bound": float(info.bound_rel_err) if prec else None,
                       "unreachable": rc == mg.ERR_TARGET_UNREACHABLE, "entries_checked": int(len(rows) * s)}
                print(json.dumps(row), file=out, flush=True)
                rows_out.append(row)
            del dA, dB, dC
            torch.cuda.empty_cache()
    return rows_out


def table(rows):
    lines = ["| s | phi | slices | used | ms | eff. FP64 TFLOP/s | max rel err (oracle) | stated bound |",
             "|---|---|---|---|---|---|---|---|"]
    for r in rows:
        # a fixed slice count states no bound (the call reports -1)
        b = "—" if r["bound"] is None or r["bound"] < 0 else (
            f"{r['bound']:.2e}" + (" (target unreachable)" if r["unreachable"] else ""))
        lines.append(f"| {r['s']} | {r['phi']} | {r['slices']} | {r['used'] or '—'} | {r['ms']:.3f} | "
                     f"{r['tflops']:.2f} | {r['err']:.2e} | {b} |")
    return "\n".join(lines)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", type=int, nargs="+", default=[2048, 4096, 8192])
    a = ap.parse_args()
    rows = sweep(a.sizes)
    print()
    print(table(rows))


if __name__ == "__main__":
    main()
