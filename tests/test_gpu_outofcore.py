"""Out-of-core calls: host operands larger than the staging budget are
computed in streamed blocks. Results are checked against the double-double
oracle with the componentwise bound 2(k+2)u(|alpha||A||B| + |beta||C0|)
(k slabs add one rounding of C per slab, well inside it), and, where the
blocking keeps k whole and the Ozaki slice count is fixed, bit for bit
against the unblocked device call."""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu

MiB = 1 << 20
U = {np.float64: 2.0**-53, np.float32: 2.0**-24}


@pytest.fixture
def budget(gpu):
    def set_(b):
        mg.check(gpu.momms_set_staging_budget(b), gpu)
    yield set_
    gpu.momms_set_staging_budget(0)


def _plan(lib, desc_like, budget_bytes):
    mb, nb, kb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    mg.check(lib.momms_stream_plan(ctypes.byref(desc_like), budget_bytes, ctypes.byref(mb), ctypes.byref(nb),
                                   ctypes.byref(kb)), lib)
    return mb.value, nb.value, kb.value


def _run(lib, A, B, C, alpha, beta, prec, budget_bytes, **kw):
    dt = mg.DTYPE_F64 if A.dtype == np.float64 else mg.DTYPE_F32
    m, k = A.shape
    n = B.shape[1]

    def trip(x):
        return (x.ctypes.data, x.strides[0] // x.itemsize, x.strides[1] // x.itemsize)

    d = gu.make_desc(dt, m, n, k, alpha, beta, trip(A), trip(B), trip(C), precision=prec, mem=mg.MEM_HOST, **kw)
    plan = _plan(lib, d, budget_bytes)
    mg.check(lib.momms_gemm(ctypes.byref(d), None), lib)
    return plan


def _bound_ok(C, A, B, C0, alpha, beta, dt):
    ref, mag = ou.dd_gemm(A.astype(np.float64), B.astype(np.float64), C0.astype(np.float64), alpha=alpha, beta=beta)
    r = ou.bound_ratio(C.astype(np.float64), ref, mag, A.shape[1], U[dt])
    assert r <= 1.0, r
    return r


CASES = [
    # dtype, precision, m, n, k, budget MiB, C layout, beta
    (np.float64, mg.PREC_PLAIN, 1500, 1300, 1100, 96, "F", 1.0),
    (np.float64, mg.PREC_PLAIN, 1000, 2100, 3000, 100, "C", -0.5),
    (np.float64, mg.PREC_OZAKI, 1536, 1280, 1024, 180, "F", 1.0),
    (np.float64, mg.PREC_OZAKI, 900, 700, 5000, 120, "F", 0.0),
    (np.float32, mg.PREC_PLAIN, 2000, 1800, 900, 90, "F", 1.0),
    (np.float32, mg.PREC_SPLIT_TF32, 1700, 1900, 1500, 110, "C", 0.25),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{np.dtype(c[0]).name}-p{c[1]}-{c[2]}x{c[3]}x{c[4]}-{c[5]}M")
def test_streamed_matches_oracle(gpu, budget, case):
    dt, prec, m, n, k, bmib, layout, beta = case
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.ascontiguousarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = np.array(rng.uniform(-1, 1, (m, n)).astype(dt), order=layout)
    C = C0.copy(order="K")
    budget(bmib * MiB)
    mb, nb, kb = _run(gpu, A, B, C, 0.75, beta, prec, bmib * MiB)
    assert (mb, nb, kb) != (m, n, k), "the budget should force blocking"
    _bound_ok(C, A, B, C0, 0.75, beta, dt)
    st = ctypes.c_uint32()
    assert gpu.momms_device_status(ctypes.byref(st)) == mg.OK and st.value == 0


def test_streamed_ozaki_fixed_slices_bitwise(gpu, budget):
    """k in one slab + a fixed slice count: every entry's digit sums are the
    same integers as in the unblocked call, so C is bit-identical."""
    rng = np.random.default_rng(77)
    m, n, k = 2048, 1792, 1024
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    ref = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI, slices=8)
    C = C0.copy(order="F")
    budget(250 * MiB)
    mb, nb, kb = _run(gpu, A, B, C, 1.0, 1.0, mg.PREC_OZAKI, 250 * MiB, slices=8)
    assert kb == k and (mb, nb) != (m, n)
    assert np.array_equal(C.view(np.uint64), ref.view(np.uint64))


def test_streamed_mixed_device_a(gpu, budget):
    """A on the device (viewed in blocks in place), B and C streamed."""
    rng = np.random.default_rng(78)
    m, n, k = 1200, 1600, 1000
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    ta, ars, acs = gu.to_device(A)
    C = C0.copy(order="F")
    d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 1.0, (ta.data_ptr(), ars, acs), (B.ctypes.data, 1, k),
                     (C.ctypes.data, 1, m))
    d.a.mem, d.b.mem, d.c.mem = mg.MEM_DEVICE, mg.MEM_HOST, mg.MEM_HOST
    budget(100 * MiB)
    assert _plan(gpu, d, 100 * MiB) != (m, n, k)
    mg.check(gpu.momms_gemm(ctypes.byref(d), None), gpu)
    _bound_ok(C, A, B, C0, 1.0, 1.0, np.float64)


def test_ozaki_k_beyond_one_launch(gpu):
    """k > 2^16 runs as k slabs (device operands), each within the target."""
    rng = np.random.default_rng(79)
    m, n, k = 256, 192, 70000
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI)
    _bound_ok(C, A, B, C0, 1.0, 1.0, np.float64)
