"""Failure detection without a GPU fault.

* Bounded waits: a self-test kernel waits on a barrier that nothing arrives
  on, with a short poll limit; it must give up, set the status bit and return,
  and the host must read MOMMS_ERR_DEVICE_TIMEOUT from the status word while
  the context stays usable.
* Host-side injection at the ABI layer: the next allocation or post-launch
  check fails the way a real failure is reported; every entry point must
  return MOMMS_ERR_OUT_OF_MEMORY / MOMMS_ERR_CUDA and the same call must then
  succeed with the same result (the library stays usable).

The reference panics on such errors (src/kern/ukernel_wrapper.rs:23-28); the
status codes tested here replace the panic.
"""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clear_faults(gpu):
    yield
    gpu.momms_fault_inject(mg.FAULT_ALLOC, 0)
    gpu.momms_fault_inject(mg.FAULT_CUDA, 0)


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("word", [0, 1])
def test_bounded_wait_expires_and_reports(gpu, word):
    read = gpu.momms_device_status if word == 0 else gpu.momms_noalloc_status
    bits = ctypes.c_uint32(0)
    assert read(ctypes.byref(bits)) == mg.OK  # clean before
    assert gpu.momms_selftest_wait_expiry(2000, word, _stream()) == mg.OK
    assert read(ctypes.byref(bits)) == mg.ERR_DEVICE_TIMEOUT
    assert bits.value & 1
    assert read(ctypes.byref(bits)) == mg.OK and bits.value == 0  # read clears it
    # the context is still usable: a GEMM runs and is right
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.uniform(-1, 1, (70, 50)))
    B = np.asfortranarray(rng.uniform(-1, 1, (50, 60)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (70, 60)))
    C = gu.gemm_device(gpu, A, B, C0)
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.bound_ratio(C, ref, mag, 50, 2.0**-53) <= 1.0


def test_selftest_rejects_bad_arguments(gpu):
    assert gpu.momms_selftest_wait_expiry(0, 0, None) == mg.ERR_INVALID_ARG
    assert gpu.momms_selftest_wait_expiry(100, 7, None) == mg.ERR_INVALID_ARG


def _operands(dt, m, n, k, seed):
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    return A, B, C0


# (name, dtype, precision, shape): every device path allocates scratch
# (split-k workspace, slice planes, TF32 planes) and launches kernels.
DEVICE_CASES = [
    ("f64 plain split-k", np.float64, mg.PREC_PLAIN, (64, 64, 20000)),
    ("f64 ozaki", np.float64, mg.PREC_OZAKI, (300, 260, 400)),
    ("f32 split-tf32", np.float32, mg.PREC_SPLIT_TF32, (300, 260, 400)),
    ("f32 ffma split-k", np.float32, mg.PREC_PLAIN, (64, 64, 20000)),
]


@pytest.mark.parametrize("kind,code", [(mg.FAULT_ALLOC, mg.ERR_OUT_OF_MEMORY), (mg.FAULT_CUDA, mg.ERR_CUDA)])
@pytest.mark.parametrize("name,dt,prec,shape", DEVICE_CASES)
def test_device_call_reports_injected_failure_then_recovers(gpu, kind, code, name, dt, prec, shape):
    import torch
    m, n, k = shape
    A, B, C0 = _operands(dt, m, n, k, len(name) * 31 + m)
    ta, ars, acs = gu.to_device(A)
    tb, brs, bcs = gu.to_device(B)
    tc, crs, ccs = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F64 if dt == np.float64 else mg.DTYPE_F32, m, n, k, 1.0, 1.0,
                     (ta.data_ptr(), ars, acs), (tb.data_ptr(), brs, bcs), (tc.data_ptr(), crs, ccs),
                     precision=prec, slices=7 if prec == mg.PREC_OZAKI else 0)
    assert gpu.momms_fault_inject(kind, 1) == mg.OK
    rc = gpu.momms_gemm(ctypes.byref(d), None)
    torch.cuda.synchronize()
    assert rc == code, (name, rc, gpu.momms_last_error())
    assert gpu.momms_fault_pending(kind) == 0
    # the same call again, from the original C: succeeds and matches a clean run
    tc.copy_(gu.to_device(C0)[0])
    mg.check(gpu.momms_gemm(ctypes.byref(d), None), gpu)
    torch.cuda.synchronize()
    C1 = tc.cpu().numpy()
    C2 = gu.gemm_device(gpu, A, B, C0, precision=prec, slices=7 if prec == mg.PREC_OZAKI else 0)
    assert np.array_equal(C1, C2)


@pytest.mark.parametrize("prec", [mg.PREC_PLAIN, mg.PREC_OZAKI])
def test_host_staged_call_reports_injected_oom_then_recovers(gpu, prec):
    A, B, C0 = _operands(np.float64, 200, 180, 150, 11)
    C = C0.copy(order="F")
    assert gpu.momms_fault_inject(mg.FAULT_ALLOC, 1) == mg.OK
    with pytest.raises(mg.MommsError) as ei:
        gu.gemm_host(gpu, A, B, C, precision=prec, slices=7 if prec == mg.PREC_OZAKI else 0)
    assert ei.value.status == mg.ERR_OUT_OF_MEMORY
    assert np.array_equal(C, C0)  # the failed call did not write C back
    gu.gemm_host(gpu, A, B, C, precision=prec, slices=7 if prec == mg.PREC_OZAKI else 0)
    C2 = gu.gemm_device(gpu, A, B, C0, precision=prec, slices=7 if prec == mg.PREC_OZAKI else 0)
    assert np.array_equal(C, C2)


@pytest.mark.parametrize("prec", [mg.PREC_PLAIN, mg.PREC_OZAKI])
def test_pack_reports_injected_oom_then_recovers(gpu, prec):
    A, _, _ = _operands(np.float64, 128, 8, 96, 5)
    ta, rs, cs = gu.to_device(A)
    src = mg.Operand(ta.data_ptr(), rs, cs, mg.MEM_DEVICE, 0)
    h = ctypes.c_void_p()
    assert gpu.momms_fault_inject(mg.FAULT_ALLOC, 1) == mg.OK
    rc = gpu.momms_pack(mg.DTYPE_F64, prec, 0, 128, 96, ctypes.byref(src), 0, None, ctypes.byref(h))
    assert rc == mg.ERR_OUT_OF_MEMORY and not h.value
    mg.check(gpu.momms_pack(mg.DTYPE_F64, prec, 0, 128, 96, ctypes.byref(src), 0, None, ctypes.byref(h)), gpu)
    assert gpu.momms_packed_bytes(h) > 0
    mg.check(gpu.momms_packed_destroy(h), gpu)


def _batch(gpu, seed, count=6):
    rng = np.random.default_rng(seed)
    descs, keep = [], []
    for i in range(count):
        dt = np.float64 if i % 2 == 0 else np.float32
        m, n, k = (int(x) for x in rng.integers(40, 300, 3))
        A, B, C0 = _operands(dt, m, n, k, seed * 100 + i)
        ta, _, _ = gu.to_device(A)
        tb, _, _ = gu.to_device(B)
        tc, _, _ = gu.to_device(C0)
        keep.append((ta, tb, tc, C0))
        descs.append(gu.make_desc(mg.DTYPE_F64 if dt == np.float64 else mg.DTYPE_F32, m, n, k, 1.0, 1.0,
                                  (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, k), (tc.data_ptr(), 1, m),
                                  mem=mg.MEM_DEVICE))
    arr = (mg.GemmDesc * count)(*descs)
    return arr, keep


@pytest.mark.parametrize("kind,code", [(mg.FAULT_ALLOC, mg.ERR_OUT_OF_MEMORY), (mg.FAULT_CUDA, mg.ERR_CUDA)])
def test_grouped_call_reports_injected_failure_then_recovers(gpu, kind, code):
    import torch
    arr, keep = _batch(gpu, 21)
    assert gpu.momms_fault_inject(kind, 1) == mg.OK
    rc = gpu.momms_gemm_grouped(arr, len(arr), None)
    torch.cuda.synchronize()
    assert rc == code, gpu.momms_last_error()
    assert gpu.momms_fault_pending(kind) == 0
    for ta, tb, tc, C0 in keep:
        tc.copy_(gu.to_device(C0)[0])
    mg.check(gpu.momms_gemm_grouped(arr, len(arr), None), gpu)
    torch.cuda.synchronize()
    for (ta, tb, tc, C0), d in zip(keep, arr):
        A = ta.cpu().numpy()
        B = tb.cpu().numpy()
        alone = gu.gemm_device(gpu, np.asfortranarray(A), np.asfortranarray(B), C0)
        assert np.array_equal(tc.cpu().numpy(), alone)


def test_plan_create_reports_injected_oom(gpu):
    arr, keep = _batch(gpu, 22)
    plan = ctypes.c_void_p()
    assert gpu.momms_fault_inject(mg.FAULT_ALLOC, 1) == mg.OK
    rc = gpu.momms_plan_create(arr, len(arr), ctypes.byref(plan))
    assert rc == mg.ERR_OUT_OF_MEMORY and not plan.value
    mg.check(gpu.momms_plan_create(arr, len(arr), ctypes.byref(plan)), gpu)
    mg.check(gpu.momms_plan_launch(plan, None), gpu)
    mg.check(gpu.momms_plan_destroy(plan), gpu)


def test_autotune_reports_injected_oom(gpu):
    A, B, C0 = _operands(np.float64, 256, 256, 2048, 8)
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F64, 256, 256, 2048, 1.0, 1.0, (ta.data_ptr(), 1, 256), (tb.data_ptr(), 1, 2048),
                     (tc.data_ptr(), 1, 256), mem=mg.MEM_DEVICE)
    res = mg.TuneResult()
    assert gpu.momms_fault_inject(mg.FAULT_ALLOC, 1) == mg.OK
    assert gpu.momms_autotune(ctypes.byref(d), ctypes.byref(res), None) == mg.ERR_OUT_OF_MEMORY
    mg.check(gpu.momms_autotune(ctypes.byref(d), ctypes.byref(res), None), gpu)
    assert res.candidates >= 1
    gpu.momms_tune_clear()


def test_served_request_reports_injected_failure_and_server_continues(gpu):
    import torch
    cfg = mg.ServerConfig(hbm_budget_bytes=4 << 30, max_batch=4, max_inflight=2, queue_capacity=64)
    srv = ctypes.c_void_p()
    mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
    try:
        A, B, C0 = _operands(np.float64, 200, 190, 300, 31)
        ta, _, _ = gu.to_device(A)
        tb, _, _ = gu.to_device(B)
        tc, _, _ = gu.to_device(C0)
        torch.cuda.synchronize()
        d = gu.make_desc(mg.DTYPE_F64, 200, 190, 300, 1.0, 1.0, (ta.data_ptr(), 1, 200), (tb.data_ptr(), 1, 300),
                         (tc.data_ptr(), 1, 200), mem=mg.MEM_DEVICE)
        assert gpu.momms_fault_inject(mg.FAULT_CUDA, 1) == mg.OK
        rid = ctypes.c_uint64()
        mg.check(gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)), gpu)
        info = mg.RequestInfo()
        gpu.momms_server_wait(srv, rid, 60.0, ctypes.byref(info))
        assert info.status == mg.ERR_CUDA
        assert gpu.momms_fault_pending(mg.FAULT_CUDA) == 0
        # the next request is served normally and equals the call alone
        tc.copy_(gu.to_device(C0)[0])
        torch.cuda.synchronize()
        mg.check(gpu.momms_server_submit(srv, ctypes.byref(d), ctypes.byref(rid)), gpu)
        mg.check(gpu.momms_server_wait(srv, rid, 60.0, ctypes.byref(info)), gpu)
        assert info.status == mg.OK
        torch.cuda.synchronize()
        assert np.array_equal(tc.cpu().numpy(), gu.gemm_device(gpu, A, B, C0))
    finally:
        mg.check(gpu.momms_server_destroy(srv), gpu)
