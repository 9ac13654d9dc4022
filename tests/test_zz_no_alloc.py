"""momms_dgemm_noalloc, the f64 entry point that allocates nothing.

It is meant for callers that cannot allocate device memory: an application
whose GPU memory already belongs to its own pool or framework, or a
latency-critical loop that cannot afford cudaMalloc / cudaFree (their cost,
their implicit synchronisation, or an out-of-memory failure midway). Its
split-k scratch is a fixed device-global array shared by every call, so each
case below runs two calls in a row. The entry point runs the same kernel with
the same tile / split-k plan as momms_dgemm, so both calls must equal
momms_dgemm bit for bit, and each must also meet the componentwise bound
against the double-double oracle directly.

The file name makes pytest collect it last: a run that stops at the first
failure has run every other test before this one.
"""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu

U64 = 2.0**-53


def _call(fn, A_t, B_t, C_t, m, n, k, alpha, beta):
    import torch
    al = ctypes.c_double(alpha)
    be = ctypes.c_double(beta)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return fn(m, n, k, ctypes.byref(al), ctypes.c_void_p(A_t.data_ptr()), A_t.stride(0), A_t.stride(1),
              ctypes.c_void_p(B_t.data_ptr()), B_t.stride(0), B_t.stride(1), ctypes.byref(be),
              ctypes.c_void_p(C_t.data_ptr()), C_t.stride(0), C_t.stride(1), s)


@pytest.mark.parametrize("shape", [(64, 64, 30000), (600, 500, 700), (1000, 1000, 300)])
def test_noalloc_matches_dgemm_twice(gpu, shape):
    import torch
    m, n, k = shape
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    A_t, _, _ = gu.to_device(A)
    B_t, _, _ = gu.to_device(B)

    ref_t, _, _ = gu.to_device(C0)
    mg.check(_call(gpu.momms_dgemm, A_t, B_t, ref_t, m, n, k, 1.0, 1.0), gpu)
    torch.cuda.synchronize()
    C_ref = ref_t.cpu().numpy()

    exact, mag = ou.dd_gemm(A, B, C0)
    for _ in range(2):  # two calls in a row: the shared scratch must not leak state
        C_t, _, _ = gu.to_device(C0)
        mg.check(_call(gpu.momms_dgemm_noalloc, A_t, B_t, C_t, m, n, k, 1.0, 1.0), gpu)
        torch.cuda.synchronize()
        C = C_t.cpu().numpy()
        assert np.array_equal(C, C_ref)  # same kernel, same plan: same bits
        assert ou.bound_ratio(C, exact, mag, k, U64) <= 1.0
    bits = ctypes.c_uint32(0)
    assert gpu.momms_noalloc_status(ctypes.byref(bits)) == mg.OK and bits.value == 0


def test_noalloc_rejects_a_plan_larger_than_its_scratch(gpu):
    """A split-k plan that needs more partial tiles than the fixed array holds
    is refused before anything runs, and C is left as it was. The model never
    plans more than one partial tile per SM; a tuning-table entry can."""
    import torch
    m, n, k = 1024, 1024, 4096  # 64 output tiles; 32 splits -> 2048 partial tiles
    rng = np.random.default_rng(404)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    A_t, _, _ = gu.to_device(A)
    B_t, _, _ = gu.to_device(B)
    C_t, _, _ = gu.to_device(C0)
    gpu.momms_tune_clear()
    mg.check(gpu.momms_tune_import(f"0 0 {m} {n} {k} 32".encode()), gpu)
    try:
        rc = _call(gpu.momms_dgemm_noalloc, A_t, B_t, C_t, m, n, k, 1.0, 1.0)
        torch.cuda.synchronize()
        assert rc == mg.ERR_INVALID_ARG
        assert b"no-alloc scratch" in gpu.momms_last_error()
        assert np.array_equal(C_t.cpu().numpy(), C0)
    finally:
        gpu.momms_tune_clear()


def test_noalloc_rejects_what_it_cannot_do_without_allocating(gpu):
    import torch
    m, n, k = 32, 32, 32
    A = np.asfortranarray(np.ones((m, k)))
    B = np.asfortranarray(np.ones((k, n)))
    C = np.asfortranarray(np.zeros((m, n)))
    al = ctypes.c_double(1.0)
    be = ctypes.c_double(0.0)
    # host operands would need staging buffers
    rc = gpu.momms_dgemm_noalloc(m, n, k, ctypes.byref(al), A.ctypes.data, 1, m, B.ctypes.data, 1, k,
                                 ctypes.byref(be), C.ctypes.data, 1, m, None)
    assert rc == mg.ERR_INVALID_ARG
    assert b"device operands" in gpu.momms_last_error()
    # general strides would need a repack copy
    big = torch.zeros((2 * m, 2 * k), dtype=torch.float64, device="cuda")
    A_t = big[::2, ::2]  # strides (4k, 2): unit along neither index
    B_t, _, _ = gu.to_device(B)
    C_t, _, _ = gu.to_device(C)
    rc = _call(gpu.momms_dgemm_noalloc, A_t, B_t, C_t, m, n, k, 1.0, 0.0)
    assert rc == mg.ERR_INVALID_ARG
    assert b"repack" in gpu.momms_last_error()
