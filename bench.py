"""Benchmark of the GB300 blocked matrix multiply (one JSON line on rank 0).

Workload (the headline of the reference's shape sweep and the FP64 target):
plain DGEMM C += A*B, m = n = k = 8192, column-major f64, entries uniform
[-1, 1] from a fixed seed, alpha = beta = 1. Every operand (512 MiB) is larger
than the 129 MB L2, so consecutive steps start cold without a flush.

  value : TFLOP/s = 2mnk / (device time per step), operands resident in HBM,
          summed over ranks (replicas) and divided by the slowest rank's time.
  e2e   : the same metric through momms_gemm() with pinned HOST operands:
          each step copies A, B and C to the device and C back.
  roofline : the DMMA kernel's achieved FP64 rate against the FP64 MMA peak
          measured in this run (momms_measure_peak).
  cpu_baseline : the reference's Goto algorithm on the host cores (the
          oracle's restatement; the reference's own asm kernels where they
          can run), on a bounded sample of the same workload.

--impl reference runs only that CPU algorithm, with every host thread, and
prints its own line.
"""
import argparse
import ctypes
import json
import math
import os
import platform
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 GEMM TFLOP/s (plain vs emulated, equal error); served GEMM p50/p99 latency"
SEED = 8192
M = N = K = 8192
WORKLOAD = "plain DGEMM C += A*B, m=n=k=8192, column-major f64, uniform[-1,1], alpha=beta=1"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--size", type=int, default=M, help="m = n = k (default 8192)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas: no data-path collective)
# ---------------------------------------------------------------------------
def dist_init(n):
    if n <= 1 or "RANK" not in os.environ:
        return 0, 1, 0
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl"
    import torch
    torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# exact sampled accuracy check (no oracle: error-free products + math.fsum)
# ---------------------------------------------------------------------------
def _two_prod(a, b):
    p = a * b
    # Veltkamp splitting (Dekker's TwoProduct), exact for |a|,|b| well inside range
    f = 134217729.0
    ah = a * f - (a * f - a)
    al = a - ah
    bh = b * f - (b * f - b)
    bl = b - bh
    e = ((ah * bh - p) + ah * bl + al * bh) + al * bl
    return p, e


def sampled_error(A, B, C0, C, samples=128, seed=7):
    """max over sampled (i, j) of |C_ij - exact_ij| / (|A||B| + |C0|)_ij."""
    rng = np.random.default_rng(seed)
    m, k = A.shape
    n = B.shape[1]
    ii = rng.integers(0, m, samples)
    jj = rng.integers(0, n, samples)
    worst = 0.0
    for i, j in zip(ii, jj):
        a = np.ascontiguousarray(A[i, :], dtype=np.float64)
        b = np.ascontiguousarray(B[:, j], dtype=np.float64)
        p, e = _two_prod(a, b)
        exact = math.fsum(np.concatenate([p, e, [float(C0[i, j])]]))
        mag = float(np.abs(p).sum()) + abs(float(C0[i, j]))
        worst = max(worst, abs(float(C[i, j]) - exact) / mag)
    return worst


# ---------------------------------------------------------------------------
# CPU reference (the reference's Goto algorithm): --impl reference and the
# cpu_baseline leg
# ---------------------------------------------------------------------------
def cpu_reference(A, B, C0, budget_s, threads):
    """Times the Goto algorithm on a row slab of the workload sized to about
    budget_s seconds. Returns (TFLOP/s, rows, seconds, kind)."""
    sys.path.insert(0, ROOT)
    from tests import oracle_util as ou
    ref = ou.load_ref()
    ukr, kind = None, "port"
    if ref is not None:
        ukr = ctypes.cast(ref.bli_dgemm_haswell_asm_6x8, ctypes.c_void_p)
        kind = "reference"
    m, k = A.shape
    n = B.shape[1]
    # calibrate on a small slab
    rows = 120
    Cs = np.asfortranarray(C0[:rows, :])
    t0 = time.perf_counter()
    ou.goto_gemm(np.asfortranarray(A[:rows, :]), B, Cs, 1.0, 1.0, threads=threads, ukr=ukr)
    dt = time.perf_counter() - t0
    rows = int(min(m, max(120, budget_s / max(dt, 1e-6) * 120)))
    rows -= rows % 120 if rows > 120 else 0
    As = np.asfortranarray(A[:rows, :])
    Cs = np.asfortranarray(C0[:rows, :])
    t0 = time.perf_counter()
    ou.goto_gemm(As, B, Cs, 1.0, 1.0, threads=threads, ukr=ukr)
    dt = time.perf_counter() - t0
    return 2.0 * rows * n * k / dt / 1e12, rows, dt, kind


def make_inputs(size):
    rng = np.random.default_rng(SEED)
    A = np.asfortranarray(rng.uniform(-1, 1, (size, size)))
    B = np.asfortranarray(rng.uniform(-1, 1, (size, size)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (size, size)))
    return A, B, C0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    size = args.size
    A, B, C0 = make_inputs(size)
    threads = os.cpu_count() or 1
    vals = []
    rows = kind = None
    for step in range(args.warmup + args.steps):
        v, rows, dt, kind = cpu_reference(A, B, C0, budget_s=4.0, threads=threads)
        if step >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    sample = f"rows 0..{rows} of C (a {rows}x{size}x{size} slab, full n and k) per step"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": f"synthetic uniform[-1,1], seed {SEED}",
            "config": {"workload": WORKLOAD.replace("8192", str(size)), "m": size, "n": size, "k": size,
                       "algorithm": "Goto NC=3000 KC=192 MC=120 + 6x8 microkernel",
                       "host": platform.machine()},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def profile_traffic(kernel_tag):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel_tag}.md")
    if not os.path.exists(path):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(path).read())
    return float(m.group(1)) if m else None


def run_ours(args):
    import torch
    import momms_gb300 as mg

    rank, world, local = dist_init(args.gpus)
    torch.cuda.set_device(local)
    lib = mg.load_library()
    size = args.size
    m = n = k = size
    flops = 2.0 * m * n * k
    A, B, C0 = make_inputs(size)

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    # device operands (column-major: a (cols, rows) tensor transposed)
    dA = torch.from_numpy(A.T.copy()).to(dev).t()
    dB = torch.from_numpy(B.T.copy()).to(dev).t()
    dC0 = torch.from_numpy(C0.T.copy()).to(dev).t()
    dC = torch.empty_like(dC0)

    def desc(a_ptr, b_ptr, c_ptr, mem):
        d = mg.GemmDesc()
        d.dtype, d.precision = mg.DTYPE_F64, mg.PREC_PLAIN
        d.m, d.n, d.k = m, n, k
        d.alpha, d.beta = 1.0, 1.0
        d.a = mg.Operand(a_ptr, 1, m, mem, 0)
        d.b = mg.Operand(b_ptr, 1, k, mem, 0)
        d.c = mg.Operand(c_ptr, 1, m, mem, 0)
        return d

    dev_desc = desc(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), mg.MEM_DEVICE)

    def step_device():
        mg.check(lib.momms_gemm(ctypes.byref(dev_desc), sp), lib)

    # C is reset from C0 before each step (a device copy, outside the per-step
    # kernel timing below; the step time is taken from events around the GEMM)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            dC.copy_(dC0)
            step_device()
        stream.synchronize()

        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        launches0 = lib.momms_launch_count()
        clocks = ClockSampler(local)
        clocks.start()
        barrier(world)
        torch.cuda.synchronize()
        t_start = time.perf_counter()
        for i in range(args.steps):
            dC.copy_(dC0)
            ev[i][0].record(stream)
            step_device()
            ev[i][1].record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_start
        clk = clocks.stop()
        launches = lib.momms_launch_count() - launches0
        step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    total_ms = max_over_ranks(total_ms, world)
    ms_per_step = total_ms / args.steps
    value = world * flops / (ms_per_step * 1e-3) / 1e12

    # accuracy of the last result on a sample of entries
    C_out = dC.t().cpu().numpy().T
    acc_err = sampled_error(A, B, C0, C_out)

    # ---- e2e through the public API with pinned host operands ----
    hA = torch.from_numpy(A.T.copy()).pin_memory().t()
    hB = torch.from_numpy(B.T.copy()).pin_memory().t()
    hC0 = torch.from_numpy(C0.T.copy()).pin_memory().t()
    hC = torch.empty((n, m), dtype=torch.float64).pin_memory().t()
    host_desc = desc(hA.data_ptr(), hB.data_ptr(), hC.data_ptr(), mg.MEM_HOST)
    e2e_steps = max(3, args.steps // 2)
    for _ in range(1):
        hC.copy_(hC0)
        mg.check(lib.momms_gemm(ctypes.byref(host_desc), sp), lib)
    barrier(world)
    e2e_t = 0.0
    for _ in range(e2e_steps):
        hC.copy_(hC0)  # host-side reset, not timed
        t0 = time.perf_counter()
        mg.check(lib.momms_gemm(ctypes.byref(host_desc), sp), lib)  # H2D A,B,C + GEMM + D2H C + sync
        e2e_t += time.perf_counter() - t0
    e2e_t = max_over_ranks(e2e_t, world)
    e2e_value = world * flops * e2e_steps / e2e_t / 1e12
    elem = 8
    h2d = 3 * m * k * elem  # A, B and C (beta = 1 reads C)
    d2h = m * n * elem

    # ---- roofline: achieved FP64 MMA rate vs the measured peak ----
    peak = ctypes.c_double(0.0)
    mg.check(lib.momms_measure_peak(0, ctypes.byref(peak)), lib)
    kernel_ms = statistics.mean(step_ms)
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    traffic = profile_traffic("dgemm_dmma_8192")

    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic: uniform[-1,1] from seed {SEED}, column-major, C initialised like A and B",
        "config": {"workload": WORKLOAD.replace("8192", str(size)), "m": m, "n": n, "k": k,
                   "precision": "plain (FP64 tensor-core MMA, mma.sync m8n8k4)",
                   "l2": "inputs larger than L2 (512 MiB per operand vs 129 MB L2); no flush",
                   "parallelism": f"replicas x{world}"},
        "accuracy": {"max_rel_err_sampled": acc_err, "definition": "max |C-exact|/(|A||B|+|C0|) over 128 entries"},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value if peak.value else None, "traffic": traffic,
                     "peak_source": "FP64 DMMA issue rate measured in this run (momms_measure_peak kind 0); "
                                    "not in MEASURED_PEAKS.json, which has HBM and bf16 only",
                     "kernel": "momms::dmma::dgemm_kernel", "algorithmic_flops_per_launch": flops},
        "e2e": {"value": e2e_value, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "api": "momms_gemm with MOMMS_MEM_HOST pinned operands"},
        "gpu_launches": int(launches),
        "clocks": clk,
        "wall_s_timed": t_wall,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, rows, dt, kind = cpu_reference(A, B, C0, budget_s=10.0, threads=threads)
        line["cpu_baseline"] = {"value": v, "unit": "TFLOP/s", "cores": threads, "kind": kind,
                                "sample": f"rows 0..{rows} of C ({rows}x{n}x{k} slab), {dt:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
