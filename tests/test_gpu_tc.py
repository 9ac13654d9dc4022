"""Parity of the tcgen05 paths with the oracle.

* split-TF32 f32 (MOMMS_PREC_SPLIT_TF32): inside the same f32 componentwise
  bound as the plain path, 2(k+2) u_32 (|alpha||A||B| + |beta||C0|).
* Ozaki FP64 emulation (MOMMS_PREC_OZAKI): exact on integer data (the whole
  slice -> tcgen05 -> int32 -> FP64 chain), error falling with the slice
  count, and the automatic slice choice meeting the requested componentwise
  error |dC_ij| / (|alpha||A||B| + |beta||C0|)_ij against the double-double
  oracle.
"""
import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu

U32 = 2.0**-24
U64 = 2.0**-53


def _mats(rng, m, n, k, dt, orders="FFF", lo=-1.0, hi=1.0):
    A = np.array(rng.uniform(lo, hi, (m, k)), dtype=dt, order=orders[0])
    B = np.array(rng.uniform(lo, hi, (k, n)), dtype=dt, order=orders[1])
    C0 = np.array(rng.uniform(lo, hi, (m, n)), dtype=dt, order=orders[2])
    return A, B, C0


# ---------------------------------------------------------------- split-TF32
@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 9, 13), (128, 256, 64), (129, 257, 100), (300, 500, 777),
                                   (1000, 17, 3000), (64, 64, 30000)])
def test_tf32x3_shapes(gpu, shape):
    m, n, k = shape
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A, B, C0 = _mats(rng, m, n, k, np.float32)
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_SPLIT_TF32)
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.bound_ratio(C, ref, mag, k, U32) <= 1.0
    # and the reference's own f32 algorithm is inside the same bound
    Cg = C0.copy(order="A")
    ou.goto_gemm(A, B, Cg)
    assert np.all(np.abs(C.astype(np.float64) - Cg) <= 4.0 * (k + 2) * U32 * mag)


@pytest.mark.parametrize("orders", ["CCC", "FCF", "CFC"])
def test_tf32x3_layouts_alpha_beta(gpu, orders):
    rng = np.random.default_rng(5)
    m, n, k = 200, 300, 150
    A, B, C0 = _mats(rng, m, n, k, np.float32, orders)
    C = gu.gemm_device(gpu, A, B, C0, 0.5, -1.25, precision=mg.PREC_SPLIT_TF32)
    ref, mag = ou.dd_gemm(A, B, C0, alpha=0.5, beta=-1.25)
    assert ou.bound_ratio(C, ref, mag, k, U32) <= 1.0


def test_tf32x3_as_accurate_as_ffma(gpu):
    """With the tensor-core accumulation promoted to FP32 registers every 256
    k, the 3-term split is about as accurate as a sequential FFMA chain."""
    rng = np.random.default_rng(9)
    A, B, C0 = _mats(rng, 512, 512, 4096, np.float32)
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_SPLIT_TF32)
    Cf = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_PLAIN)
    ref, mag = ou.dd_gemm(A, B, C0)
    e_tc, e_ffma = ou.rel_err(C, ref, mag), ou.rel_err(Cf, ref, mag)
    assert e_tc <= 4 * e_ffma, (e_tc, e_ffma)


# ---------------------------------------------------------------- Ozaki
def test_ozaki_integer_data_is_exact(gpu):
    """Small integers fit one digit: the product must be exact."""
    rng = np.random.default_rng(1)
    m, n, k = 300, 260, 1000
    A = np.asfortranarray(rng.integers(-8, 9, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-8, 9, (k, n)).astype(np.float64))
    C0 = np.asfortranarray(rng.integers(-100, 100, (m, n)).astype(np.float64))
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI, slices=1)
    exact = C0 + (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(C, exact)


def test_ozaki_two_digit_integers_exact(gpu):
    """Entries up to 2^12 need at most two digits; with s = 3 the kept pairs
    (t + u <= 4) include every nonzero product, so the result is exact."""
    rng = np.random.default_rng(2)
    m, n, k = 129, 257, 700
    A = np.asfortranarray(rng.integers(-4000, 4001, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(-4000, 4001, (k, n)).astype(np.float64))
    C0 = np.zeros((m, n), order="F")
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI, slices=3)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(C, exact)


def test_ozaki_full_digit_chunks_exact(gpu):
    """One 8-bit digit per entry (values 200..255, one sign): every TMEM
    chunk of the top x top pair (4 k-blocks of 64) sums to within 1 % of
    the 2^24 bound with arbitrary low bits; the result must be exact."""
    rng = np.random.default_rng(12)
    m, n, k = 256, 320, 8192
    A = np.asfortranarray(rng.integers(200, 256, (m, k)).astype(np.float64))
    B = np.asfortranarray(rng.integers(200, 256, (k, n)).astype(np.float64))
    C0 = np.zeros((m, n), order="F")
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI, slices=1)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(C, exact)


def test_ozaki_top_by_centred_chunks_exact(gpu):
    """Values 256 t + 128 (t in 200..254) split into a top digit t + 1 and a
    centred digit -128: the top x centred chunks (8 k-blocks) reach 99.6 %
    of the 2^24 bound, all of one sign; with 3 slices every nonzero digit
    product is kept, so the result must be exact."""
    rng = np.random.default_rng(13)
    m, n, k = 192, 256, 4096
    A = np.asfortranarray((256 * rng.integers(200, 255, (m, k)) + 128).astype(np.float64))
    B = np.asfortranarray((256 * rng.integers(200, 255, (k, n)) + 128).astype(np.float64))
    C0 = np.zeros((m, n), order="F")
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI, slices=3)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(C, exact)


def test_ozaki_error_falls_with_slices(gpu):
    rng = np.random.default_rng(3)
    m, n, k = 256, 256, 512
    A, B, C0 = _mats(rng, m, n, k, np.float64)
    ref, mag = ou.dd_gemm(A, B, C0)
    errs = []
    for s in range(2, 10):
        C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI, slices=s)
        errs.append(ou.rel_err(C, ref, mag))
    for a, b in zip(errs, errs[1:]):
        assert b <= a * 1.01 or b < 4 * U64
    assert errs[0] > 1e-6  # 2 slices: about 14 bits
    assert errs[-1] < 4 * U64  # 9 slices: FP64 level


@pytest.mark.parametrize("phi", [0.5, 2.0, 8.0])
def test_ozaki_auto_slices_meet_target(gpu, phi):
    """Inputs of the emulation sweep: a = U[-0.5,0.5] * exp(phi N(0,1))."""
    rng = np.random.default_rng(int(phi * 10))
    m, n, k = 192, 320, 300
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, k)) * np.exp(phi * rng.standard_normal((m, k))))
    B = np.asfortranarray(rng.uniform(-0.5, 0.5, (k, n)) * np.exp(phi * rng.standard_normal((k, n))))
    C0 = np.zeros((m, n), order="F")
    ref, mag = ou.dd_gemm(A, B, C0, beta=0.0)
    for target in (1e-8, 1e-12):
        C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI, target_rel_err=target)
        # the bound is worst case: the measured error must sit below the target
        # (plus the final FP64 rounding of C)
        assert ou.rel_err(C, ref, mag) <= target + 4 * U64


@pytest.mark.parametrize("orders", ["FFF", "CCC", "CFC"])
def test_ozaki_layouts_alpha_beta_fp64_level(gpu, orders):
    rng = np.random.default_rng(4)
    m, n, k = 333, 211, 390
    A, B, C0 = _mats(rng, m, n, k, np.float64, orders)
    C = gu.gemm_device(gpu, A, B, C0, -0.75, 0.5, precision=mg.PREC_OZAKI)
    ref, mag = ou.dd_gemm(A, B, C0, alpha=-0.75, beta=0.5)
    # default target: FP64 level; also inside the plain-path bound
    assert ou.bound_ratio(C, ref, mag, k, U64) <= 1.0
    assert ou.rel_err(C, ref, mag) < 8 * U64


def test_ozaki_small_and_ragged(gpu):
    rng = np.random.default_rng(6)
    for (m, n, k) in [(1, 1, 1), (7, 9, 13), (130, 258, 65)]:
        A, B, C0 = _mats(rng, m, n, k, np.float64)
        C = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI)
        ref, mag = ou.dd_gemm(A, B, C0)
        assert ou.bound_ratio(C, ref, mag, k, U64) <= 1.0


def test_ozaki_nonfinite_rows_propagate(gpu):
    rng = np.random.default_rng(8)
    m, n, k = 40, 30, 20
    A, B, C0 = _mats(rng, m, n, k, np.float64)
    A[5, 3] = np.nan
    B[2, 7] = np.inf
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI)
    assert np.all(np.isnan(C[5, :]))
    assert np.all(np.isnan(C[:, 7]))
    mask = np.ones_like(C, dtype=bool)
    mask[5, :] = False
    mask[:, 7] = False
    assert np.all(np.isfinite(C[mask]))


def test_ozaki_deterministic(gpu):
    rng = np.random.default_rng(10)
    A, B, C0 = _mats(rng, 300, 300, 300, np.float64)
    C1 = gu.gemm_device(gpu, A, B, C0, precision=mg.PREC_OZAKI)
    C2 = gu.gemm_device(gpu, A, B, C0, precision=mg.PREC_OZAKI)
    assert np.array_equal(C1, C2)


def test_no_bounded_wait_expired(gpu):
    """No kernel of the tcgen05 paths gave up on a barrier during this module."""
    import ctypes
    rng = np.random.default_rng(12)
    A, B, C0 = _mats(rng, 1000, 1000, 2000, np.float64)
    gu.gemm_device(gpu, A, B, C0, precision=mg.PREC_OZAKI)
    A32, B32, C32 = (x.astype(np.float32) for x in (A, B, C0))
    gu.gemm_device(gpu, np.asfortranarray(A32), np.asfortranarray(B32), np.asfortranarray(C32),
                   precision=mg.PREC_SPLIT_TF32)
    bits = ctypes.c_uint32(0)
    assert gpu.momms_device_status(ctypes.byref(bits)) == mg.OK, bits.value
    assert bits.value == 0


# ------------------------------------------------------- operand passes, layouts
def _device_view(X, kind, rng):
    """A device tensor holding X's values in the given layout: "col" / "row"
    (contiguous), "offset" (a view one element past an aligned start, leading
    dimension odd: rows never 16-byte aligned), "strided" (neither stride 1)."""
    import torch
    r, c = X.shape
    t = torch.from_numpy(np.ascontiguousarray(X))
    if kind == "col":
        return t.t().contiguous().t().cuda()
    if kind == "row":
        return t.cuda()
    if kind == "offset":
        ld = r + 3 if (r + 3) % 2 else r + 4
        big = torch.zeros((c * ld + 1,), dtype=t.dtype).cuda()
        v = torch.as_strided(big, (r, c), (1, ld), storage_offset=1)
        v.copy_(t.cuda())
        return v
    if kind == "strided":
        big = torch.zeros((2 * r, 3 * c), dtype=t.dtype).cuda()
        v = big[::2, ::3]
        v.copy_(t.cuda())
        return v
    raise ValueError(kind)


def _run_views(lib, A, B, C0, prec, a_kind, b_kind):
    import ctypes
    import torch
    m, k = A.shape
    n = B.shape[1]
    dt = mg.DTYPE_F64 if A.dtype == np.float64 else mg.DTYPE_F32
    ta, tb = _device_view(A, a_kind, None), _device_view(B, b_kind, None)
    tc = torch.from_numpy(np.asfortranarray(C0).T.copy()).cuda().t()  # column-major C
    d = gu.make_desc(dt, m, n, k, 0.5, -1.0, (ta.data_ptr(), ta.stride(0), ta.stride(1)),
                     (tb.data_ptr(), tb.stride(0), tb.stride(1)), (tc.data_ptr(), tc.stride(0), tc.stride(1)),
                     precision=prec)
    mg.check(lib.momms_gemm(ctypes.byref(d), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), lib)
    torch.cuda.synchronize()
    return tc.cpu().numpy()


@pytest.mark.parametrize("prec", [mg.PREC_OZAKI, mg.PREC_SPLIT_TF32])
@pytest.mark.parametrize("shape", [(257, 190, 203), (300, 45, 5), (7000, 40, 24)])
def test_operand_passes_layout_independent(gpu, prec, shape):
    """Row maxima, magnitudes and digit planes depend only on the values, so
    the result is bit-identical whatever layout the operands arrive in: rows
    contiguous or not, rows not 16-byte aligned (scalar loads), neither
    stride 1, rows of a few elements (several rows per warp), many rows."""
    rng = np.random.default_rng(hash(shape) % 2**32)
    m, n, k = shape
    dt = np.float64 if prec == mg.PREC_OZAKI else np.float32
    A, B, C0 = _mats(rng, m, n, k, dt)
    ref = _run_views(gpu, A, B, C0, prec, "col", "col")
    for a_kind, b_kind in [("row", "row"), ("offset", "offset"), ("strided", "strided"), ("row", "offset"),
                           ("offset", "strided")]:
        C = _run_views(gpu, A, B, C0, prec, a_kind, b_kind)
        assert np.array_equal(C, ref), (a_kind, b_kind)
    exact, mag = ou.dd_gemm(A.astype(np.float64), B.astype(np.float64), C0.astype(np.float64), alpha=0.5, beta=-1.0)
    assert ou.bound_ratio(ref, exact, mag, k, U64 if dt == np.float64 else U32) <= 1.0


def test_ozaki_rows_past_one_launch_of_row_maxima(gpu):
    """Row maxima of a column-major A run in launches of 65535 x 32 rows: a
    2.2 M-row A (row scales spread over 2^-30..2^30, so a wrong row exponent
    shows) is inside the FP64-level bound on every entry, rows past the first
    launch included."""
    rng = np.random.default_rng(22)
    m, n, k = 2_200_000, 8, 8
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)) * np.exp2(rng.integers(-30, 31, m))[:, None])
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    C = gu.gemm_device(gpu, A, B, C0, 1.0, 0.5, precision=mg.PREC_OZAKI)
    ref, mag = ou.dd_gemm(A, B, C0, alpha=1.0, beta=0.5)
    assert ou.bound_ratio(C, ref, mag, k, U64) <= 1.0
    assert ou.bound_ratio(C[65535 * 32:], ref[65535 * 32:], mag[65535 * 32:], k, U64) <= 1.0
