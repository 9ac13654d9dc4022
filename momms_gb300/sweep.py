"""Shape sweep over the measurement configurations of the path (device-resident
operands, CUDA events, warm-up first):

  * square s x s x s for s in 256 .. 8192: f64 plain, f64 emulated (Ozaki),
    f32 plain (FFMA), f32 split-TF32
  * rank-k m = n = 8192, k in {64, 256} and tall-skinny 65536 x 256 x 256:
    achieved HBM GB/s and the fraction of min(peak FLOP/s, intensity x HBM),
    since these shapes can be memory-bound
  * emulated FP64 on a_ij = U[-0.5, 0.5] * exp(phi * N(0, 1)) for phi in
    {0.5, 2, 8} at 2048 / 4096 / 8192: slice count chosen per call, sampled
    error against error-free products, effective FP64 TFLOP/s vs plain DGEMM

    python -m momms_gb300.sweep [--quick] > sweep.jsonl

One JSON line per configuration. Errors are max over sampled entries of
|C_ij - exact_ij| / (|A||B|)_ij (exact by two-product splitting and math.fsum).
"""
import argparse
import ctypes
import json
import math
import os
import sys

import numpy as np

import momms_gb300 as mg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _two_prod(a, b):
    """Error-free products a*b = p + e (Dekker/Veltkamp splitting)."""
    p = a * b
    split = 134217729.0  # 2^27 + 1
    ca = split * a
    ah = ca - (ca - a)
    al = a - ah
    cb = split * b
    bh = cb - (cb - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def sampled_error(A, B, C, samples=48, seed=11):
    rng = np.random.default_rng(seed)
    m, k = A.shape
    n = B.shape[1]
    worst = 0.0
    for i, j in zip(rng.integers(0, m, samples), rng.integers(0, n, samples)):
        a = np.ascontiguousarray(A[i, :], dtype=np.float64)
        b = np.ascontiguousarray(B[:, j], dtype=np.float64)
        p, e = _two_prod(a, b)
        exact = math.fsum(np.concatenate([p, e]))
        mag = float(np.abs(p).sum())
        if not math.isfinite(float(C[i, j])):
            return math.inf
        if mag > 0:
            worst = max(worst, abs(float(C[i, j]) - exact) / mag)
    return worst


def peaks(lib):
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    mp = json.load(open(path)) if os.path.exists(path) else {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    f64 = ctypes.c_double()
    f32 = ctypes.c_double()
    mg.check(lib.momms_measure_peak(0, ctypes.byref(f64)), lib)
    mg.check(lib.momms_measure_peak(1, ctypes.byref(f32)), lib)
    return {"hbm_gbs": mp["hbm_gbs"], "f16_tflops": mp["bf16_tflops"], "tf32_tflops": mp["bf16_tflops"] / 2,
            "f64_tflops": f64.value, "f32_tflops": f32.value}


def run_one(lib, torch, dtype, prec, m, n, k, phi=None, reps=3, warmup=1, err=False):
    tdt = torch.float64 if dtype == "f64" else torch.float32
    g = torch.Generator(device="cuda").manual_seed(m * 31 + n * 7 + k)

    def make(rows, cols):
        # column-major rows x cols
        if phi is None:
            x = torch.rand((cols, rows), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
        else:
            u = torch.rand((cols, rows), dtype=torch.float64, device="cuda", generator=g) - 0.5
            x = u * torch.exp(phi * torch.randn((cols, rows), dtype=torch.float64, device="cuda", generator=g))
        return x.to(tdt).t()

    A, B = make(m, k), make(k, n)
    C = torch.zeros((n, m), dtype=tdt, device="cuda").t()
    d = mg.GemmDesc()
    d.dtype = mg.DTYPE_F64 if dtype == "f64" else mg.DTYPE_F32
    d.precision = prec
    d.m, d.n, d.k = m, n, k
    d.alpha, d.beta = 1.0, 0.0
    d.a = mg.Operand(A.data_ptr(), 1, m, mg.MEM_DEVICE, 0)
    d.b = mg.Operand(B.data_ptr(), 1, k, mg.MEM_DEVICE, 0)
    d.c = mg.Operand(C.data_ptr(), 1, m, mg.MEM_DEVICE, 0)
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    for _ in range(warmup):
        mg.check(lib.momms_gemm(ctypes.byref(d), sp), lib)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        mg.check(lib.momms_gemm(ctypes.byref(d), sp), lib)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    info = mg.CallInfo()
    lib.momms_last_info(ctypes.byref(info))
    out = {"dtype": dtype, "prec": {0: "plain", 1: "ozaki", 2: "tf32"}[prec], "m": m, "n": n, "k": k, "ms": ms,
           "tflops": 2.0 * m * n * k / (ms * 1e-3) / 1e12}
    if prec == mg.PREC_OZAKI:
        out["slices"] = info.slices
        out["pairs"] = info.pairs
        out["bound_rel_err"] = info.bound_rel_err
    if phi is not None:
        out["phi"] = phi
    if err:
        Cn = C.double().cpu().numpy()
        out["err"] = sampled_error(A.double().cpu().numpy(), B.double().cpu().numpy(), Cn)
        out["nonfinite"] = int((~np.isfinite(Cn)).sum())
        out["c_absmax"] = float(np.abs(Cn[np.isfinite(Cn)]).max()) if np.isfinite(Cn).any() else 0.0
    return out


def roofline(o, pk):
    """Adds achieved GB/s (A, B and C once each) and, where the work per
    product is known, the bound min(peak, intensity x HBM) in FP64/f32
    TFLOP/s of the call and the fraction reached. Emulated FP64 runs
    `pairs` fp16 slice products per output product, so its peak is the fp16
    rate divided by the pair count."""
    es = 8 if o["dtype"] == "f64" else 4
    m, n, k = o["m"], o["n"], o["k"]
    bytes_ = es * (m * k + k * n + m * n)  # beta = 0: C written once
    flops = 2.0 * m * n * k
    ozaki_peak = pk["f16_tflops"] / o["pairs"] if o.get("pairs") else None
    peak = {"plain": pk["f64_tflops"] if o["dtype"] == "f64" else pk["f32_tflops"],
            "ozaki": ozaki_peak, "tf32": pk["tf32_tflops"] / 3}[o["prec"]]
    o["gbs"] = bytes_ / (o["ms"] * 1e-3) / 1e9
    if peak is not None:
        bound = min(peak, flops / bytes_ * pk["hbm_gbs"] / 1e3)
        o["bound_tflops"] = bound
        o["frac_of_bound"] = o["tflops"] / bound
    return o


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="skip 8192^3 plain f64 (1 s per call)")
    ap.add_argument("--only", choices=["square", "shapes", "phi"], default=None)
    a = ap.parse_args()
    import torch
    lib = mg.load_library()
    pk = peaks(lib)
    print(json.dumps({"peaks": pk}), flush=True)
    sizes = [256, 512, 1024, 2048, 4096, 8192] if a.only in (None, "square") else []
    for s in sizes:
        for dtype, prec in (("f64", mg.PREC_PLAIN), ("f64", mg.PREC_OZAKI), ("f32", mg.PREC_PLAIN),
                            ("f32", mg.PREC_SPLIT_TF32)):
            if a.quick and s == 8192 and dtype == "f64" and prec == mg.PREC_PLAIN:
                continue
            reps = 2 if (dtype == "f64" and prec == mg.PREC_PLAIN and s >= 4096) else 5
            print(json.dumps(roofline(run_one(lib, torch, dtype, prec, s, s, s, reps=reps), pk)), flush=True)
    shapes = ((8192, 8192, 64), (8192, 8192, 256), (65536, 256, 256)) if a.only in (None, "shapes") else ()
    for (m, n, k) in shapes:
        for dtype, prec in (("f64", mg.PREC_PLAIN), ("f64", mg.PREC_OZAKI), ("f32", mg.PREC_PLAIN),
                            ("f32", mg.PREC_SPLIT_TF32)):
            print(json.dumps(roofline(run_one(lib, torch, dtype, prec, m, n, k, reps=5), pk)), flush=True)
    for s in ((2048, 4096, 8192) if a.only in (None, "phi") else ()):
        for phi in (0.5, 2.0, 8.0):
            o = run_one(lib, torch, "f64", mg.PREC_OZAKI, s, s, s, phi=phi, reps=3, err=True)
            print(json.dumps(o), flush=True)
        if not (a.quick and s == 8192):
            o = run_one(lib, torch, "f64", mg.PREC_PLAIN, s, s, s, phi=2.0, reps=1, err=True)
            print(json.dumps(o), flush=True)


if __name__ == "__main__":
    sys.exit(main())
