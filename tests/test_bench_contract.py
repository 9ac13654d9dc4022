"""bench.py on the CPU: the reference arm's JSON line with the keys a driver
reads, under torchrun a line from rank 0 only (the other ranks exit 0
without work), and the replicas' timing plumbing (barrier, max over ranks)
on two gloo ranks."""
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
