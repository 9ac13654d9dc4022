"""Run one GEMM configuration repeatedly on the GPU (timing and profiling aid).

    python -m momms_gb300.run --m 4096 --n 4096 --k 4096 --dtype f64 --prec ozaki --reps 3
    python -m momms_gb300.run --batched 512 --reps 5

Operands are device-resident, column-major, uniform [-1, 1] from a fixed
seed; C starts equal to A*B-sized random data and beta = 1. Prints one JSON
line with the mean device time per call (CUDA events) and TFLOP/s.

--batched N runs the uneven batch of the grouped-launch measurement instead:
N problems with m, n, k log-uniform over [32, 1024] (numpy seed 512), half
f64 and half f32, plain, as one execution plan launched through its CUDA
graph.
"""
import argparse
import ctypes
import json

import momms_gb300 as mg


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--m", type=int, default=4096)
    p.add_argument("--n", type=int, default=4096)
    p.add_argument("--k", type=int, default=4096)
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64")
    p.add_argument("--prec", choices=["plain", "ozaki", "tf32"], default="plain")
    p.add_argument("--slices", type=int, default=0)
    p.add_argument("--target", type=float, default=0.0)
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=1)
    p.add_argument("--kernels", action="store_true",
                   help="also report each kernel class's mean time per call (CUDA events per launch)")
    p.add_argument("--batched", type=int, default=0, help="time a plan of this many uneven problems instead")
    p.add_argument("--tune", action="store_true", help="with --batched: autotune every shape bucket first")
    a = p.parse_args()
    if a.batched:
        return run_batched(a)

    import torch
    lib = mg.load_library()
    dt = torch.float64 if a.dtype == "f64" else torch.float32
    g = torch.Generator(device="cuda").manual_seed(1234)
    A = (torch.rand((a.k, a.m), dtype=dt, device="cuda", generator=g) * 2 - 1).t()
    B = (torch.rand((a.n, a.k), dtype=dt, device="cuda", generator=g) * 2 - 1).t()
    C = (torch.rand((a.n, a.m), dtype=dt, device="cuda", generator=g) * 2 - 1).t()
    d = mg.GemmDesc()
    d.dtype = mg.DTYPE_F64 if a.dtype == "f64" else mg.DTYPE_F32
    d.precision = {"plain": mg.PREC_PLAIN, "ozaki": mg.PREC_OZAKI, "tf32": mg.PREC_SPLIT_TF32}[a.prec]
    d.m, d.n, d.k = a.m, a.n, a.k
    d.alpha, d.beta = 1.0, 1.0
    d.a = mg.Operand(A.data_ptr(), 1, a.m, mg.MEM_DEVICE, 0)
    d.b = mg.Operand(B.data_ptr(), 1, a.k, mg.MEM_DEVICE, 0)
    d.c = mg.Operand(C.data_ptr(), 1, a.m, mg.MEM_DEVICE, 0)
    d.slices = a.slices
    d.target_rel_err = a.target
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    for _ in range(a.warmup):
        mg.check(lib.momms_gemm(ctypes.byref(d), sp), lib)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(a.reps):
        mg.check(lib.momms_gemm(ctypes.byref(d), sp), lib)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(1, a.reps)
    info = mg.CallInfo()
    lib.momms_last_info(ctypes.byref(info))
    out = {"m": a.m, "n": a.n, "k": a.k, "dtype": a.dtype, "prec": a.prec, "ms": ms,
           "tflops": 2.0 * a.m * a.n * a.k / (ms * 1e-3) / 1e12, "slices": info.slices,
           "pairs": info.pairs, "splits": info.splits, "slice_variant": info.slice_variant}
    if a.kernels:
        # separate timed pass: per-launch events would perturb the whole-call time above
        lib.momms_timing_enable(1)
        for _ in range(a.reps):
            mg.check(lib.momms_gemm(ctypes.byref(d), sp), lib)
        torch.cuda.synchronize()
        names = {mg.KERNEL_DGEMM_DMMA: "dgemm_dmma", mg.KERNEL_SGEMM_FFMA: "sgemm_ffma",
                 mg.KERNEL_SLICE_OZAKI: "slice_ozaki", mg.KERNEL_SLICE_TF32: "slice_tf32",
                 mg.KERNEL_PREP: "prep", mg.KERNEL_COMBINE: "combine", mg.KERNEL_BOUND: "bound"}
        per = {}
        for cls, name in names.items():
            tot, cnt = ctypes.c_double(), ctypes.c_ulonglong()
            lib.momms_timing_read(cls, ctypes.byref(tot), ctypes.byref(cnt), 1)
            if cnt.value:
                per[name] = tot.value / a.reps
        lib.momms_timing_enable(0)
        out["kernel_ms_per_call"] = per
    print(json.dumps(out))


def run_batched(a):
    """The grouped-launch batch: one plan, captured, relaunched `reps` times."""
    import numpy as np
    import torch
    lib = mg.load_library()
    rng = np.random.default_rng(512)
    kinds = rng.choice(3, a.batched, p=[0.5, 0.0, 0.5])
    dims = np.exp(rng.uniform(np.log(32), np.log(1024), (a.batched, 3))).astype(np.int64)
    descs = (mg.GemmDesc * a.batched)()
    keep = []
    flops = 0.0
    for i in range(a.batched):
        m, n, k = (int(x) for x in dims[i])
        dt = torch.float32 if kinds[i] == 2 else torch.float64
        A = (torch.rand((k, m), dtype=dt, device="cuda") * 2 - 1).t()
        B = (torch.rand((n, k), dtype=dt, device="cuda") * 2 - 1).t()
        C = (torch.rand((n, m), dtype=dt, device="cuda") * 2 - 1).t()
        d = mg.GemmDesc()
        d.dtype = mg.DTYPE_F32 if kinds[i] == 2 else mg.DTYPE_F64
        d.precision = mg.PREC_PLAIN
        d.m, d.n, d.k = m, n, k
        d.alpha, d.beta = 1.0, 1.0
        d.a = mg.Operand(A.data_ptr(), 1, m, mg.MEM_DEVICE, 0)
        d.b = mg.Operand(B.data_ptr(), 1, k, mg.MEM_DEVICE, 0)
        d.c = mg.Operand(C.data_ptr(), 1, m, mg.MEM_DEVICE, 0)
        descs[i] = d
        keep.append((A, B, C))
        flops += 2.0 * m * n * k
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    lib.momms_tune_clear()
    tuned = ctypes.c_int32(0)
    if a.tune:
        mg.check(lib.momms_autotune_batch(descs, a.batched, sp, ctypes.byref(tuned)), lib)
    plan = ctypes.c_void_p()
    mg.check(lib.momms_plan_create(descs, a.batched, ctypes.byref(plan)), lib)
    # per-kernel split from uncaptured launches
    lib.momms_timing_enable(1)
    for kc in (mg.KERNEL_DGEMM_DMMA, mg.KERNEL_SGEMM_FFMA):
        lib.momms_timing_read(kc, None, None, 1)
    for _ in range(max(1, a.reps)):
        mg.check(lib.momms_plan_launch(plan, sp), lib)
    split = {}
    for kc, name in ((mg.KERNEL_DGEMM_DMMA, "f64_kernel_ms"), (mg.KERNEL_SGEMM_FFMA, "f32_kernel_ms")):
        t = ctypes.c_double(0)
        n_ = ctypes.c_ulonglong(0)
        lib.momms_timing_read(kc, ctypes.byref(t), ctypes.byref(n_), 1)
        split[name] = t.value / max(1, a.reps)
    lib.momms_timing_enable(0)
    mg.check(lib.momms_plan_capture(plan, sp), lib)
    for _ in range(a.warmup):
        mg.check(lib.momms_plan_launch(plan, sp), lib)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(a.reps):
        mg.check(lib.momms_plan_launch(plan, sp), lib)
    e1.record(s)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / max(1, a.reps)
    lib.momms_plan_destroy(plan)
    f64_flops = sum(2.0 * float(dims[i][0] * dims[i][1] * dims[i][2]) for i in range(a.batched) if kinds[i] != 2)
    out = {"batched": a.batched, "f64_problems": int((kinds != 2).sum()), "f32_problems": int((kinds == 2).sum()),
           "ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "tuned_buckets": tuned.value, **split}
    if split.get("f64_kernel_ms"):
        out["f64_tflops"] = f64_flops / (split["f64_kernel_ms"] * 1e-3) / 1e12
    if split.get("f32_kernel_ms"):
        out["f32_tflops"] = (flops - f64_flops) / (split["f32_kernel_ms"] * 1e-3) / 1e12
    lib.momms_tune_clear()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
