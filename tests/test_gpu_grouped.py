"""Grouped persistent launches, execution plans with CUDA graphs, autotuning.

A problem is planned from its own shape only, so each result of a batch must
be bit-identical to the same problem run alone through momms_gemm.
"""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu


def _logu(rng, lo, hi, size):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size)).astype(np.int64)


def _batch(rng, count, lo=32, hi=512, precisions=None):
    """Device operands for `count` problems: half f64, half f32 (plain unless
    `precisions` says otherwise). Returns (descs, tensors, host copies)."""
    import torch
    dims = np.stack([_logu(rng, lo, hi, count) for _ in range(3)], axis=1)
    descs = (mg.GemmDesc * count)()
    keep, host = [], []
    for i, (m, n, k) in enumerate(dims):
        m, n, k = int(m), int(n), int(k)
        f64 = i % 2 == 0
        dt = np.float64 if f64 else np.float32
        A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
        B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
        C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
        ta, ars, acs = gu.to_device(A)
        tb, brs, bcs = gu.to_device(B)
        tc, crs, ccs = gu.to_device(C0)
        prec = precisions[i] if precisions else mg.PREC_PLAIN
        d = gu.make_desc(mg.DTYPE_F64 if f64 else mg.DTYPE_F32, m, n, k, 1.0, 1.0, (ta.data_ptr(), ars, acs),
                         (tb.data_ptr(), brs, bcs), (tc.data_ptr(), crs, ccs), precision=prec, mem=mg.MEM_DEVICE,
                         slices=6 if prec == mg.PREC_OZAKI else 0)
        descs[i] = d
        keep.append((ta, tb, tc))
        host.append((A, B, C0))
    return descs, keep, host


def _single(gpu, d, A, B, C0):
    """The same problem alone through momms_gemm on fresh device copies."""
    import torch
    ta, ars, acs = gu.to_device(A)
    tb, brs, bcs = gu.to_device(B)
    tc, crs, ccs = gu.to_device(C0)
    d2 = gu.make_desc(d.dtype, d.m, d.n, d.k, d.alpha, d.beta, (ta.data_ptr(), ars, acs), (tb.data_ptr(), brs, bcs),
                      (tc.data_ptr(), crs, ccs), precision=d.precision, mem=mg.MEM_DEVICE, slices=d.slices)
    mg.check(gpu.momms_gemm(ctypes.byref(d2), None), gpu)
    torch.cuda.synchronize()
    return tc.cpu().numpy()


def test_grouped_bitwise_equals_single(gpu):
    import torch
    rng = np.random.default_rng(2024)
    descs, keep, host = _batch(rng, 48)
    mg.check(gpu.momms_gemm_grouped(descs, len(descs), None), gpu)
    torch.cuda.synchronize()
    for i in range(len(descs)):
        C = keep[i][2].cpu().numpy()
        A, B, C0 = host[i]
        Cs = _single(gpu, descs[i], A, B, C0)
        assert np.array_equal(C, Cs), i
    # and inside the componentwise bound
    for i in range(0, len(descs), 7):
        A, B, C0 = host[i]
        C = keep[i][2].cpu().numpy()
        ref, mag = ou.dd_gemm(A, B, C0)
        u = 2.0**-53 if A.dtype == np.float64 else 2.0**-24
        assert ou.bound_ratio(C, ref, mag, A.shape[1], u) <= 1.0


def test_plan_graph_relaunch_and_mixed_modes(gpu):
    import torch
    rng = np.random.default_rng(7)
    n = 12
    precs = [mg.PREC_PLAIN] * n
    precs[2] = mg.PREC_OZAKI  # f64
    precs[5] = mg.PREC_SPLIT_TF32  # f32
    descs, keep, host = _batch(rng, n, lo=64, hi=400, precisions=precs)
    plan = ctypes.c_void_p()
    mg.check(gpu.momms_plan_create(descs, n, ctypes.byref(plan)), gpu)
    mg.check(gpu.momms_plan_capture(plan, None), gpu)
    expected = [_single(gpu, descs[i], *host[i]) for i in range(n)]
    for rep in range(2):
        for i in range(n):  # reset C in place (the plan keeps the pointers)
            keep[i][2].copy_(torch.from_numpy(np.ascontiguousarray(host[i][2].T)).t())
        mg.check(gpu.momms_plan_launch(plan, None), gpu)
        torch.cuda.synchronize()
        for i in range(n):
            assert np.array_equal(keep[i][2].cpu().numpy(), expected[i]), (rep, i)
    mg.check(gpu.momms_plan_destroy(plan), gpu)


def test_plan_rejects_host_operands(gpu):
    A = np.asfortranarray(np.ones((8, 8)))
    d = gu.make_desc(mg.DTYPE_F64, 8, 8, 8, 1.0, 0.0, (A.ctypes.data, 1, 8), (A.ctypes.data, 1, 8),
                     (A.ctypes.data, 1, 8), mem=mg.MEM_HOST)
    arr = (mg.GemmDesc * 1)(d)
    plan = ctypes.c_void_p()
    assert gpu.momms_plan_create(arr, 1, ctypes.byref(plan)) == mg.ERR_INVALID_ARG


def test_autotune_records_and_keeps_c(gpu):
    import torch
    rng = np.random.default_rng(3)
    m, n, k = 96, 80, 6000  # few tiles, long k: split-k candidates matter
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 1.0, (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, k),
                     (tc.data_ptr(), 1, m), mem=mg.MEM_DEVICE)
    gpu.momms_tune_clear()
    res = mg.TuneResult()
    mg.check(gpu.momms_autotune(ctypes.byref(d), ctypes.byref(res), None), gpu)
    assert res.candidates >= 2 and 1 <= res.splits <= 32 and res.best_ms > 0
    assert np.array_equal(tc.cpu().numpy(), C0)  # tuning writes only scratch
    need = ctypes.c_size_t(0)
    gpu.momms_tune_export(None, 0, ctypes.byref(need))
    buf = ctypes.create_string_buffer(need.value)
    mg.check(gpu.momms_tune_export(buf, need.value, None), gpu)
    line = buf.value.decode().strip()
    # keyed by the shape's bucket, written as the bucket's largest shape
    assert line == f"0 0 128 128 8192 {res.splits} {res.tile}"
    # the tuned plan is used and the result is still inside the bound
    mg.check(gpu.momms_gemm(ctypes.byref(d), None), gpu)
    torch.cuda.synchronize()
    info = mg.CallInfo()
    gpu.momms_last_info(ctypes.byref(info))
    assert info.splits == res.splits
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.bound_ratio(tc.cpu().numpy(), ref, mag, k, 2.0**-53) <= 1.0
    gpu.momms_tune_clear()


def test_emulated_problems_share_one_slice_launch(gpu):
    """A plan's emulated problems (uneven sizes, one of a single 128-row tile,
    different slice counts) run their slice products in one persistent
    launch, with each result bit-identical to the problem alone; the captured
    plan relaunches with the same bits."""
    import torch
    rng = np.random.default_rng(31)
    shapes = [(700, 520, 300), (96, 300, 257), (1030, 900, 640), (256, 256, 64), (333, 129, 1000)]
    slices = [7, 6, 8, 5, 7]
    descs = (mg.GemmDesc * len(shapes))()
    keep, host = [], []
    for i, ((m, n, k), s) in enumerate(zip(shapes, slices)):
        A = np.asfortranarray(rng.uniform(-1, 1, (m, k)) * np.exp(rng.standard_normal((m, k))))
        B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
        C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
        ta, ars, acs = gu.to_device(A)
        tb, brs, bcs = gu.to_device(B)
        tc, crs, ccs = gu.to_device(C0)
        descs[i] = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0 if i % 2 else -0.5, 1.0, (ta.data_ptr(), ars, acs),
                                (tb.data_ptr(), brs, bcs), (tc.data_ptr(), crs, ccs), precision=mg.PREC_OZAKI,
                                mem=mg.MEM_DEVICE, slices=s)
        keep.append((ta, tb, tc))
        host.append((A, B, C0))
    expected = [_single(gpu, descs[i], *host[i]) for i in range(len(shapes))]
    plan = ctypes.c_void_p()
    mg.check(gpu.momms_plan_create(descs, len(shapes), ctypes.byref(plan)), gpu)
    gpu.momms_timing_enable(1)
    gpu.momms_timing_read(mg.KERNEL_SLICE_OZAKI, None, None, 1)
    mg.check(gpu.momms_plan_launch(plan, None), gpu)
    torch.cuda.synchronize()
    launches = ctypes.c_ulonglong(0)
    gpu.momms_timing_read(mg.KERNEL_SLICE_OZAKI, None, ctypes.byref(launches), 1)
    gpu.momms_timing_enable(0)
    assert launches.value == 1  # one slice launch for all five problems
    for i in range(len(shapes)):
        assert np.array_equal(keep[i][2].cpu().numpy(), expected[i]), i
    mg.check(gpu.momms_plan_capture(plan, None), gpu)
    for rep in range(2):
        for i in range(len(shapes)):
            keep[i][2].copy_(torch.from_numpy(np.ascontiguousarray(host[i][2].T)).t())
        mg.check(gpu.momms_plan_launch(plan, None), gpu)
        torch.cuda.synchronize()
        for i in range(len(shapes)):
            assert np.array_equal(keep[i][2].cpu().numpy(), expected[i]), (rep, i)
    mg.check(gpu.momms_plan_destroy(plan), gpu)
