"""Full-matrix parity at the configurations the benchmark and the sweep report.

Every entry of C is checked against the double-double oracle (no sampling):

* rank-k updates m = n = 8192 with k = 64 and 256, and the tall-skinny
  65536 x 256 x 256 shape, in all four modes (f64 on DMMA, f64 emulated from
  fp16 slices, f32 on FFMA, f32 as split TF32);
* square 2048^3 in all four modes;
* the emulation inputs a = U[-0.5,0.5] exp(phi N(0,1)) at 2048^3 for
  phi = 0.5, 2, 8: fixed slice counts 3..9 (error falling as slices are
  added) and the automatic count at a 1e-14 target, met on every entry or
  reported unreachable with a bound that holds;
* one FFMA call whose operand offsets pass 2^32 elements (the kernel's 64-bit
  offset path).

Bounds: plain f64 and f32 within |dC_ij| <= 2(k+2) u (|A||B| + |C0|)_ij (u the
unit roundoff of the type; the reference's own check is the Freivalds
residual, src/util.rs:55-85); the emulated results within the bound the call
reports (momms_last_info), which holds for every entry.
"""
import ctypes
import functools

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu

U64 = 2.0**-53
U32 = 2.0**-24

MODES = [("f64", mg.PREC_PLAIN), ("f64", mg.PREC_OZAKI), ("f32", mg.PREC_PLAIN), ("f32", mg.PREC_SPLIT_TF32)]
SHAPES = [(8192, 8192, 64), (8192, 8192, 256), (65536, 256, 256), (2048, 2048, 2048)]


@functools.lru_cache(maxsize=2)
def _problem(shape, dt):
    """Operands (uniform[-1, 1], C initialised like A and B, as the benchmark)
    and the oracle's exact result for alpha = beta = 1."""
    m, n, k = shape
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    ref, mag = ou.dd_gemm(A, B, C0)
    return A, B, C0, ref, mag


def _device_call(gpu, A, B, C0, precision, **kw):
    import torch
    m, k = A.shape
    n = B.shape[1]
    dt = mg.DTYPE_F64 if A.dtype == np.float64 else mg.DTYPE_F32
    ta, ars, acs = gu.to_device(A)
    tb, brs, bcs = gu.to_device(B)
    tc, crs, ccs = gu.to_device(C0)
    d = gu.make_desc(dt, m, n, k, 1.0, 1.0, (ta.data_ptr(), ars, acs), (tb.data_ptr(), brs, bcs),
                     (tc.data_ptr(), crs, ccs), precision=precision, **kw)
    rc = gpu.momms_gemm(ctypes.byref(d), None)
    torch.cuda.synchronize()
    info = mg.CallInfo()
    gpu.momms_last_info(ctypes.byref(info))
    return rc, tc.cpu().numpy(), info


MODE_NAMES = {(("f64", mg.PREC_PLAIN)): "f64", ("f64", mg.PREC_OZAKI): "ozaki", ("f32", mg.PREC_PLAIN): "f32",
              ("f32", mg.PREC_SPLIT_TF32): "tf32x3"}
# grouped by shape, f64 modes before f32 ones, so that each oracle result is
# computed once (the cache holds the f64 and the f32 problem of one shape)
CASES = [pytest.param(shape, dtype, prec, id=f"{'x'.join(map(str, shape))}-{MODE_NAMES[(dtype, prec)]}")
         for shape in SHAPES for (dtype, prec) in MODES]


@pytest.mark.parametrize("shape,dtype,precision", CASES)
def test_full_matrix_parity(gpu, shape, dtype, precision):
    dt = np.float64 if dtype == "f64" else np.float32
    A, B, C0, ref, mag = _problem(shape, dt)
    rc, C, info = _device_call(gpu, A, B, C0, precision)
    assert rc == mg.OK, gpu.momms_last_error()
    k = shape[2]
    if precision == mg.PREC_OZAKI:
        # the bound the call states holds for every entry (plus C's FP64
        # rounding and the beta update)
        assert 0.0 < info.bound_rel_err <= 2.0**-52
        assert ou.rel_err(C, ref, mag) <= info.bound_rel_err + 4 * U64
    else:
        assert ou.bound_ratio(C, ref, mag, k, U64 if dt == np.float64 else U32) <= 1.0


@functools.lru_cache(maxsize=1)
def _spread_problem(phi):
    n = 2048
    rng = np.random.default_rng(int(phi * 100) + 7)
    A = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, n)) * np.exp(phi * rng.standard_normal((n, n))))
    B = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, n)) * np.exp(phi * rng.standard_normal((n, n))))
    C0 = np.zeros((n, n), order="F")
    ref, mag = ou.dd_gemm(A, B, C0, beta=0.0)
    return A, B, C0, ref, mag


@pytest.mark.parametrize("phi", [0.5, 2.0, 8.0])
def test_emulation_inputs_slice_sweep_and_automatic_count(gpu, phi):
    A, B, C0, ref, mag = _spread_problem(phi)
    errs = []
    for s in range(3, 10):
        rc, C, info = _device_call(gpu, A, B, C0, mg.PREC_OZAKI, slices=s)
        assert rc == mg.OK and info.slices == s
        errs.append(ou.rel_err(C, ref, mag))
    for a, b in zip(errs, errs[1:]):
        assert b <= a, errs  # never worse with one more slice
        # once the digits reach every entry's terms (wide spreads leave some
        # entries without any at 3-4 slices), 8 more bits are far better until
        # FP64 rounding is all that is left
        if 8 * U64 < a < 1e-3:
            assert b < a / 16, errs
    rc, C, info = _device_call(gpu, A, B, C0, mg.PREC_OZAKI, target_rel_err=1e-14)
    err = ou.rel_err(C, ref, mag)
    if rc == mg.ERR_TARGET_UNREACHABLE:
        # wide spreads (phi = 8: about 2^80 between a row's largest and
        # smallest entries) put entries out of reach of per-row / per-column
        # power-of-two scaling: the call says so, with the 15-slice result and
        # the bound that holds for it
        assert info.slices == 15 and info.bound_rel_err > 1e-14
        assert err <= info.bound_rel_err + 4 * U64
        print(f"phi={phi}: target unreachable, bound {info.bound_rel_err:.3g}, measured {err:.3g}")
    else:
        assert rc == mg.OK, gpu.momms_last_error()
        assert info.bound_rel_err <= 1e-14
        assert err <= 1e-14
        print(f"phi={phi}: {info.slices} slices, bound {info.bound_rel_err:.3g}, measured {err:.3g}")


def test_ffma_offsets_beyond_32_bits(gpu):
    """A's column stride puts its last column more than 2^32 elements past its
    first, so the FFMA kernel takes its 64-bit offset path (about 17.6 GB of
    device memory hold the view)."""
    import torch
    m, n, k = 256, 192, 128
    cs = (1 << 25) + (1 << 20)
    assert (k - 1) * cs + m > 2**32
    rng = np.random.default_rng(77)
    A = rng.uniform(-1, 1, (m, k)).astype(np.float32)
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)).astype(np.float32))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(np.float32))
    big = torch.empty((k - 1) * cs + m, dtype=torch.float32, device="cuda")
    Av = torch.as_strided(big, (m, k), (1, cs))
    Av.copy_(torch.from_numpy(A))
    tb, brs, bcs = gu.to_device(B)
    tc, crs, ccs = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F32, m, n, k, 1.0, 1.0, (Av.data_ptr(), 1, cs), (tb.data_ptr(), brs, bcs),
                     (tc.data_ptr(), crs, ccs), mem=mg.MEM_DEVICE)
    mg.check(gpu.momms_gemm(ctypes.byref(d), None), gpu)
    torch.cuda.synchronize()
    C = tc.cpu().numpy()
    del big, Av
    torch.cuda.empty_cache()
    ref, mag = ou.dd_gemm(np.asfortranarray(A), B, C0)
    assert ou.bound_ratio(C, ref, mag, k, U32) <= 1.0


def test_slice_sweep_script_small(gpu):
    """tests/slice_sweep.py at 512^3, phi = 2: every entry checked; the error
    never grows with a slice added, and the automatic count's stated bound
    holds."""
    from tests import slice_sweep
    rows = slice_sweep.sweep([512], phis=(2.0,), slice_range=range(3, 7), out=open("/dev/null", "w"))
    fixed = [r for r in rows if r["slices"].isdigit()]
    assert [r["used"] for r in fixed] == [3, 4, 5, 6]
    errs = [r["err"] for r in fixed]
    assert all(b <= a for a, b in zip(errs, errs[1:])), errs
    auto = rows[-1]
    assert auto["slices"].startswith("auto") and auto["err"] <= auto["bound"] + 4 * U64
    assert all(r["entries_checked"] == 512 * 512 for r in rows)
    assert "| 512 | 2.0 | auto 1e-14 |" in slice_sweep.table(rows)
