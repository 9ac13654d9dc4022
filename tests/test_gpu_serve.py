"""The serving loop: continuous batching under an HBM admission budget.

Each served result must be bit-identical to the same request run alone
through momms_gemm (plain f64, Ozaki f64 at a 1e-14 target, plain f32), while
requests that arrive during earlier batches are admitted and launched before
those batches finish.
"""
import ctypes
import threading
import time

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu


def _request(rng, kind, lo=64, hi=700):
    """(desc, tensors, host copies) for one request of `kind`."""
    m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(lo), np.log(hi), 3)))
    dt = np.float32 if kind == "f32" else np.float64
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    prec = {"f64": mg.PREC_PLAIN, "ozaki": mg.PREC_OZAKI, "f32": mg.PREC_PLAIN}[kind]
    d = gu.make_desc(mg.DTYPE_F32 if kind == "f32" else mg.DTYPE_F64, m, n, k, 1.0, 1.0, (ta.data_ptr(), 1, m),
                     (tb.data_ptr(), 1, k), (tc.data_ptr(), 1, m), precision=prec, mem=mg.MEM_DEVICE,
                     target_rel_err=1e-14 if kind == "ozaki" else 0.0)
    return d, (ta, tb, tc), (A, B, C0)


def _alone(gpu, d, A, B, C0):
    import torch
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    d2 = gu.make_desc(d.dtype, d.m, d.n, d.k, d.alpha, d.beta, (ta.data_ptr(), 1, d.m), (tb.data_ptr(), 1, d.k),
                      (tc.data_ptr(), 1, d.m), precision=d.precision, mem=mg.MEM_DEVICE,
                      target_rel_err=d.target_rel_err)
    mg.check(gpu.momms_gemm(ctypes.byref(d2), None), gpu)
    torch.cuda.synchronize()
    return tc.cpu().numpy()


def test_served_results_equal_alone_and_batches_overlap(gpu):
    import torch
    rng = np.random.default_rng(55)
    kinds = ["f64", "ozaki", "f64", "ozaki", "f32"] * 8  # 40 / 40 / 20 %
    reqs = [_request(rng, kind) for kind in kinds]
    cfg = mg.ServerConfig(hbm_budget_bytes=8 << 30, max_batch=8, max_inflight=2, queue_capacity=1024)
    srv = ctypes.c_void_p()
    mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
    ids = []
    # two bursts: the second arrives while the first is on the GPU
    for i, (d, _, _) in enumerate(reqs):
        rid = ctypes.c_uint64(0)
        mg.check(gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)), gpu)
        ids.append(rid.value)
        if i == len(reqs) // 2:
            time.sleep(0.002)
    infos = []
    for rid in ids:
        info = mg.RequestInfo()
        mg.check(gpu.momms_server_wait(srv, rid, 60.0, ctypes.byref(info)), gpu)
        infos.append((info.submit_s, info.start_s, info.done_s, info.batch_size, info.batch_id,
                      info.device_start_ms, info.device_end_ms))
    rep = mg.ServerReport()
    mg.check(gpu.momms_server_stats(srv, ctypes.byref(rep), 0), gpu)
    assert rep.completed == len(reqs) and rep.failed == 0 and rep.rejected == 0
    assert rep.batches >= 2 and rep.p50_ms > 0 and rep.p99_ms >= rep.p50_ms
    # continuous batching: two launches' device intervals (CUDA events on
    # their streams around each launch) intersect, so their work overlapped
    # on the GPU
    batches = sorted({(x[4], x[5], x[6]) for x in infos})
    assert len(batches) == rep.batches and all(0 <= s < e for _, s, e in batches)
    overlapping = [(a, b) for i, a in enumerate(batches) for b in batches[i + 1:]
                   if max(a[1], b[1]) < min(a[2], b[2])]
    assert overlapping, batches
    mg.check(gpu.momms_server_destroy(srv), gpu)
    torch.cuda.synchronize()
    for (d, t, h) in reqs:
        served = t[2].cpu().numpy()
        alone = _alone(gpu, d, *h)
        assert np.array_equal(served, alone)


def test_admission_and_errors(gpu):
    import torch
    rng = np.random.default_rng(56)
    d, t, h = _request(rng, "f64", 200, 300)
    cfg = mg.ServerConfig(hbm_budget_bytes=1 << 20, max_batch=4, max_inflight=1, queue_capacity=2)
    srv = ctypes.c_void_p()
    mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
    rid = ctypes.c_uint64(0)
    assert gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)) == mg.ERR_ADMISSION
    A = np.asfortranarray(np.ones((4, 4)))
    dh = gu.make_desc(mg.DTYPE_F64, 4, 4, 4, 1.0, 0.0, (A.ctypes.data, 1, 4), (A.ctypes.data, 1, 4),
                      (A.ctypes.data, 1, 4), mem=mg.MEM_HOST)
    assert gpu.momms_server_submit(srv, ctypes.byref(dh), ctypes.byref(rid)) == mg.ERR_INVALID_ARG
    rep = mg.ServerReport()
    mg.check(gpu.momms_server_stats(srv, ctypes.byref(rep), 1), gpu)
    assert rep.rejected == 1
    mg.check(gpu.momms_server_destroy(srv), gpu)


def test_budget_holds_back_but_completes(gpu):
    """A budget that fits one request at a time still serves all of them, in order."""
    import torch
    rng = np.random.default_rng(57)
    reqs = [_request(rng, "f32", 300, 400) for _ in range(6)]
    one = max(4 * (r[0].m * r[0].k + r[0].k * r[0].n + r[0].m * r[0].n) for r in reqs) + (21 << 20)
    cfg = mg.ServerConfig(hbm_budget_bytes=int(one * 1.5), max_batch=8, max_inflight=2, queue_capacity=64)
    srv = ctypes.c_void_p()
    mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
    ids = []
    for d, _, _ in reqs:
        rid = ctypes.c_uint64(0)
        mg.check(gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)), gpu)
        ids.append(rid.value)
    mg.check(gpu.momms_server_drain(srv, 60.0), gpu)
    rep = mg.ServerReport()
    mg.check(gpu.momms_server_stats(srv, ctypes.byref(rep), 0), gpu)
    assert rep.completed == 6 and rep.mean_batch == 1.0 and rep.batches == 6
    for rid in ids:
        assert gpu.momms_server_poll(srv, rid, None) == mg.OK
    mg.check(gpu.momms_server_destroy(srv), gpu)


def test_emulated_requests_of_a_batch_share_one_slice_launch(gpu):
    """Emulated requests submitted together land in one batch, whose plan runs
    their slice products in one persistent launch; each result still equals
    the request run alone."""
    import torch
    rng = np.random.default_rng(71)
    reqs = [_request(rng, "ozaki", lo=200, hi=600) for _ in range(6)]
    expected = [_alone(gpu, d, *host) for d, _, host in reqs]
    cfg = mg.ServerConfig(hbm_budget_bytes=8 << 30, max_batch=16, max_inflight=1, queue_capacity=64)
    srv = ctypes.c_void_p()
    gpu.momms_timing_enable(1)
    gpu.momms_timing_read(mg.KERNEL_SLICE_OZAKI, None, None, 1)
    gpu.momms_timing_read(mg.KERNEL_BOUND, None, None, 1)
    # the server starts with the queue already full: one batch takes all six
    mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
    ids = []
    for d, _, _ in reqs:
        rid = ctypes.c_uint64(0)
        mg.check(gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)), gpu)
        ids.append(rid.value)
    mg.check(gpu.momms_server_drain(srv, 60.0), gpu)
    batches = set()
    for rid in ids:
        info = mg.RequestInfo()
        mg.check(gpu.momms_server_poll(srv, rid, ctypes.byref(info)), gpu)
        assert info.status == mg.OK
        batches.add(info.batch_id)
    mg.check(gpu.momms_server_destroy(srv), gpu)
    torch.cuda.synchronize()
    slice_launches = ctypes.c_ulonglong(0)
    gpu.momms_timing_read(mg.KERNEL_SLICE_OZAKI, None, ctypes.byref(slice_launches), 1)
    gpu.momms_timing_enable(0)
    # one slice launch per batch (the slice-count choice at plan creation
    # runs the bound kernel per problem, counted in its own class)
    assert slice_launches.value == len(batches) < len(reqs)
    for (d, dev, host), exp in zip(reqs, expected):
        assert np.array_equal(dev[2].cpu().numpy(), exp)
