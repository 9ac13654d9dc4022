"""The fused emulated-FP64 kernel against the unfused path.

For small k the slice products and the recombination of their exact sums run
in one kernel (the sums stay in registers instead of int32 planes in HBM).
It forms the same exact 128-bit integer per entry and rounds it the same way,
so its results must equal the unfused path's bit for bit at every fixed slice
count, layout, alpha and beta; MOMMS_OZAKI_FUSED=0 / 1 selects the path.
"""
import ctypes
import os

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu


def _run(gpu, A, B, C0, alpha, beta, fused, **kw):
    old = os.environ.get("MOMMS_OZAKI_FUSED")
    os.environ["MOMMS_OZAKI_FUSED"] = "1" if fused else "0"
    try:
        C = gu.gemm_device(gpu, A, B, C0, alpha, beta, precision=mg.PREC_OZAKI, **kw)
        info = mg.CallInfo()
        mg.check(gpu.momms_last_info(ctypes.byref(info)), gpu)
    finally:
        if old is None:
            del os.environ["MOMMS_OZAKI_FUSED"]
        else:
            os.environ["MOMMS_OZAKI_FUSED"] = old
    return C, info


@pytest.mark.parametrize("shape,orders,alpha,beta", [
    ((1000, 900, 64), "FFF", 1.0, 1.0),
    ((777, 1300, 300), "FFF", -0.75, 0.5),
    ((640, 515, 129), "CFC", 1.0, 0.0),
    ((300, 260, 2048), "FCF", 2.0, -1.0),
])
@pytest.mark.parametrize("slices", [3, 7, 8, 12])
def test_fused_equals_unfused(gpu, shape, orders, alpha, beta, slices):
    m, n, k = shape
    rng = np.random.default_rng(m + n + k + slices)

    def mat(r, c, o):
        x = rng.uniform(-1, 1, (r, c)) * np.exp(rng.standard_normal((r, c)))
        return np.asfortranarray(x) if o == "F" else np.ascontiguousarray(x)

    A, B, C0 = mat(m, k, orders[0]), mat(k, n, orders[1]), mat(m, n, orders[2])
    Cu, iu = _run(gpu, A, B, C0, alpha, beta, False, slices=slices)
    Cf, inf_ = _run(gpu, A, B, C0, alpha, beta, True, slices=slices)
    assert inf_.slice_variant == 3 and iu.slice_variant != 3
    assert np.array_equal(Cf, Cu)
    if slices >= 7:
        ref, mag = ou.dd_gemm(A, B, C0, alpha, beta)
        assert ou.rel_err(Cf, ref, mag) <= (1e-12 if slices == 7 else 1e-14)


def test_fused_nan_rows_and_columns(gpu):
    rng = np.random.default_rng(3)
    m, n, k = 400, 300, 128
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    A[17, 5] = np.nan
    B[9, 250] = np.inf
    Cu, _ = _run(gpu, A, B, C0, 1.0, 1.0, False, slices=7)
    Cf, info = _run(gpu, A, B, C0, 1.0, 1.0, True, slices=7)
    assert info.slice_variant == 3
    assert np.all(np.isnan(Cf[17, :])) and np.all(np.isnan(Cf[:, 250]))
    assert np.array_equal(Cf, Cu, equal_nan=True)


def test_fused_is_the_default_for_small_k_and_host_operands_stay_correct(gpu):
    """Automatic choice at small k runs the fused kernel; a host-staged call
    (its count verified before C is written) keeps the unfused recombination;
    both meet the target."""
    rng = np.random.default_rng(8)
    m, n, k = 1024, 1100, 64
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    C = gu.gemm_device(gpu, A, B, C0, precision=mg.PREC_OZAKI, target_rel_err=1e-14)
    info = mg.CallInfo()
    mg.check(gpu.momms_last_info(ctypes.byref(info)), gpu)
    assert info.slice_variant == 3
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.rel_err(C, ref, mag) <= 1e-14
    Ch = C0.copy(order="F")
    gu.gemm_host(gpu, A, B, Ch, precision=mg.PREC_OZAKI, target_rel_err=1e-14)
    assert ou.rel_err(Ch, ref, mag) <= 1e-14
