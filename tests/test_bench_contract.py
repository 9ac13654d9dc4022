"""bench.py on the CPU: the reference arm's JSON line with the keys a driver
reads, under torchrun a line from rank 0 only (the other ranks exit 0
without work), the replicas' timing plumbing (barrier, max over ranks) on
two gloo ranks, and the helpers behind the clocks, roofline.traffic and
accuracy keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _json_lines(out):
    lines = []
    for line in out.splitlines():
        line = line.strip()
        if line.startswith("{"):
            lines.append(json.loads(line))
    return lines


def _check_line(d, n_gpus):
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "dtype", "data"):
        assert isinstance(d[key], str) and d[key]
    assert d["n_gpus"] == n_gpus and d["steps"] == 1 and d["warmup"] == 1
    assert d["higher_is_better"] is True and d["scaling"] in ("weak", "strong")
    assert d["value"] > 0 and d["vs_baseline"] is None
    assert "workload" in d["config"] and d["config"]["m"] == 256
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--size", "256"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_line(lines[0], 1)


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29517", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1", "--size", "256"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check_line(lines[0], 2)


def _rank_worker(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        # each rank's timed total differs; every rank must see the slowest
        results[rank] = bench.max_over_ranks(1.5 * (rank + 1), world)
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    """The replicas' timing plumbing of bench.py (barrier, max over ranks) on
    two gloo ranks: both ranks get the larger of the two totals."""
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        results = mgr.dict()
        procs = [ctx.Process(target=_rank_worker, args=(r, 2, 29531, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=300)
            assert p.exitcode == 0
        assert dict(results) == {0: 3.0, 1: 3.0}
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(2.5, 1) == 2.5


def _bench():
    sys.path.insert(0, ROOT)
    import bench
    return bench


class _DoneProc:
    """Stands in for the nvidia-smi process once its lines are in."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_sampler_keeps_the_timed_window():
    """The clocks key: median SM clock of the samples inside the timed window
    (one period of slack at the end), the max clock, and every throttle
    reason seen active there; samples outside the window do not count."""
    bench = _bench()
    s = bench.ClockSampler(0)
    s.proc = _DoneProc()
    na, act = "Not Active", "Active"

    def ln(sm, reasons):
        return f"0, {sm}, 2070, 1100.5, 0x0, {reasons[0]}, {reasons[1]}, {reasons[2]}, {reasons[3]}"
    s.lines = [(0.50, ln(2070, (na, na, na, na))),           # before the window
               (1.00, ln(1800, (na, na, na, act))),
               (1.20, ln(1700, (na, na, na, act))),
               (1.40, ln(1750, (na, na, na, na))),
               (1.54, ln(1650, (na, na, na, na))),           # inside the slack after t1
               (2.00, ln(1000, (act, na, na, na)))]          # after the window
    out = s.stop(1.0, 1.5)
    assert out["samples"] == 4 and out["sm_mhz"] == 1725.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    # a window shorter than the period takes the first sample after it starts
    s2 = bench.ClockSampler(0)
    s2.proc = _DoneProc()
    s2.lines = [(0.9, ln(2000, (na,) * 4)), (1.3, ln(1900, (na, na, act, na)))]
    out = s2.stop(1.0, 1.01)
    assert out["samples"] == 1 and out["sm_mhz"] == 1900.0 and out["reasons"] == ["sw_thermal_slowdown"]
    # no nvidia-smi: the key says so
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_profile_traffic_reads_the_committed_summaries():
    """roofline.traffic comes from the ncu summaries under profiles/."""
    bench = _bench()
    for tag in ("slice_gemm_ozaki_8192", "dgemm_dmma_8192"):
        t = bench.profile_traffic(tag)
        assert t is not None and 1e9 < t < 1e12, tag
    assert bench.profile_traffic("no_such_profile") is None


def test_sampled_error_is_exact_and_catches_a_wrong_entry():
    """The accuracy key: zero on data whose products and sums are exact in
    FP64, and the relative size of a planted error in one sampled entry."""
    import numpy as np
    bench = _bench()
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.integers(-8, 9, (64, 40)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-8, 9, (40, 48)).astype(np.float64))
    C0 = np.asfortranarray(rng.integers(-8, 9, (64, 48)).astype(np.float64))
    C = C0 + A @ B
    assert bench.sampled_error(A, B, C0, C, samples=4000) == 0.0
    bad = C.copy()
    bad[:, :] += 1e-6 * (np.abs(A) @ np.abs(B) + np.abs(C0))
    err = bench.sampled_error(A, B, C0, bad, samples=64)
    assert 0.5e-6 < err < 2e-6
