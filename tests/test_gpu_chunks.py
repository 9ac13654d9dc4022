"""Column-chunked emulated calls: an Ozaki call may cut n into column chunks
whose B preparation, slice products and recombination run on two streams,
with B and C copied in from host memory chunk by chunk (the slice count is
chosen from B's sampled columns, copied first). Every entry's exact sums do
not depend on the cut, so every chunk count, every operand placement and the
unchunked device call give the same bits. MOMMS_OZAKI_CHUNKS fixes the count."""
import os

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu


@pytest.fixture
def chunks():
    old = os.environ.get("MOMMS_OZAKI_CHUNKS")

    def set_(v):
        os.environ["MOMMS_OZAKI_CHUNKS"] = str(v)

    yield set_
    if old is None:
        os.environ.pop("MOMMS_OZAKI_CHUNKS", None)
    else:
        os.environ["MOMMS_OZAKI_CHUNKS"] = old


def _bits(x):
    return x.view(np.uint64)


@pytest.mark.parametrize("b_order,c_order", [("F", "F"), ("C", "C"), ("F", "C")])
def test_chunk_counts_agree(gpu, chunks, b_order, c_order):
    rng = np.random.default_rng(77 + len(b_order + c_order))
    m, n, k = 700, 2600, 900  # ragged last chunk; cuts at multiples of 256 columns
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.array(rng.uniform(-1, 1, (k, n)) * np.exp2(rng.integers(-20, 20, (1, n))), order=b_order)
    C0 = np.array(rng.uniform(-1, 1, (m, n)), order=c_order)
    chunks(1)
    ref = gu.gemm_device(gpu, A, B, C0, 0.75, -1.5, precision=mg.PREC_OZAKI)
    for nch in (2, 3, 5, 8):
        chunks(nch)
        got = gu.gemm_device(gpu, A, B, C0, 0.75, -1.5, precision=mg.PREC_OZAKI)
        assert np.array_equal(_bits(got), _bits(ref)), f"device, {nch} chunks"
        C = C0.copy(order="K")
        gu.gemm_host(gpu, A, B, C, 0.75, -1.5, precision=mg.PREC_OZAKI)
        assert np.array_equal(_bits(C), _bits(ref)), f"host, {nch} chunks"
    ii, jj = rng.integers(0, m, 256), rng.integers(0, n, 256)
    exact, mag = ou.dd_gemm_entries(A, B, C0, ii, jj, 0.75, -1.5)
    assert ou.rel_err(ref[ii, jj], exact, mag) < 2.0 ** -50


@pytest.mark.parametrize("nch", [1, 4])
def test_host_chunks_beta_zero_and_fixed_slices(gpu, chunks, nch):
    """beta == 0 (C is not copied in), and a fixed slice count (no sampled
    columns copied ahead)."""
    rng = np.random.default_rng(5 + nch)
    m, n, k = 512, 4096, 640
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    chunks(1)
    refs = [gu.gemm_device(gpu, A, B, C0, 1.0, 0.0, precision=mg.PREC_OZAKI),
            gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI, slices=5)]
    chunks(nch)
    C = C0.copy(order="F")
    C[:] = np.nan  # not read with beta == 0
    gu.gemm_host(gpu, A, B, C, 1.0, 0.0, precision=mg.PREC_OZAKI)
    assert np.array_equal(_bits(C), _bits(refs[0]))
    C = C0.copy(order="F")
    gu.gemm_host(gpu, A, B, C, 1.0, 1.0, precision=mg.PREC_OZAKI, slices=5)
    assert np.array_equal(_bits(C), _bits(refs[1]))


def test_default_chunks_large_host_call(gpu):
    """The default policy chunks a 2048 x 8192 x 2048 host call (n >= 4096,
    operands from host memory); the result equals the device call's."""
    rng = np.random.default_rng(21)
    m, n, k = 2048, 8192, 2048
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    os.environ.pop("MOMMS_OZAKI_CHUNKS", None)
    ref = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI)
    C = C0.copy(order="F")
    gu.gemm_host(gpu, A, B, C, 1.0, 1.0, precision=mg.PREC_OZAKI)
    assert np.array_equal(_bits(C), _bits(ref))
    ii, jj = rng.integers(0, m, 256), rng.integers(0, n, 256)
    exact, mag = ou.dd_gemm_entries(A, B, C0, ii, jj)
    assert ou.rel_err(C[ii, jj], exact, mag) < 2.0 ** -50


def test_long_k_host_staged(gpu, chunks):
    """k above one launch's range: deferred B and C arrive whole before the
    k slabs; same bits as the device call."""
    rng = np.random.default_rng(3)
    m, n, k = 64, 300, 70000
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    chunks(1)
    ref = gu.gemm_device(gpu, A, B, C0, 1.0, 1.0, precision=mg.PREC_OZAKI)
    C = C0.copy(order="F")
    gu.gemm_host(gpu, A, B, C, 1.0, 1.0, precision=mg.PREC_OZAKI)
    assert np.array_equal(_bits(C), _bits(ref))
