"""Host-staged calls: momms_gemm with host operands copies them in on a copy
stream while the kernels that do not need them yet run, and copies C back per
column range. The kernels are the same as for device operands, so every
result must be bit-identical to the all-device call, for every precision, C
layout (column-major, row-major, sub-view, general strides: the host-scatter
fallback), beta == 0 (C not read) and mixed host/device operands."""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

MODES = [(np.float64, mg.PREC_PLAIN), (np.float64, mg.PREC_OZAKI), (np.float32, mg.PREC_PLAIN),
         (np.float32, mg.PREC_SPLIT_TF32)]


def _c_layout(rng, m, n, dt, layout):
    if layout == "F":
        return np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    if layout == "C":
        return np.ascontiguousarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    if layout == "sub":  # leading dimension larger than m
        big = np.asfortranarray(rng.uniform(-1, 1, (m + 9, n + 3)).astype(dt))
        return big[5:5 + m, 2:2 + n]
    big = np.asfortranarray(rng.uniform(-1, 1, (2 * m, n)).astype(dt))  # general strides
    return big[::2, :]


@pytest.mark.parametrize("mode", MODES, ids=["f64", "ozaki", "f32", "tf32"])
@pytest.mark.parametrize("layout", ["F", "C", "sub", "gen"])
@pytest.mark.parametrize("beta", [0.0, -0.75])
def test_host_staged_matches_device(gpu, mode, layout, beta):
    dt, prec = mode
    rng = np.random.default_rng(abs(hash((layout, beta, prec))) % 2**32)
    m, n, k = 300, 517, 260
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.ascontiguousarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = _c_layout(rng, m, n, dt, layout)
    ref = gu.gemm_device(gpu, A, B, C0, 1.25, beta, precision=prec)
    if layout in ("F", "C"):
        C = C0.copy(order="K")
    else:  # keep the strided view: operate on a fresh copy of the parent
        parent = np.array(C0.base, copy=True, order="F")
        C = parent[5:5 + m, 2:2 + n] if layout == "sub" else parent[::2, :]
        before = parent.copy()
    gu.gemm_host(gpu, A, B, C, 1.25, beta, precision=prec)
    assert np.array_equal(C.view(np.uint64 if dt == np.float64 else np.uint32),
                          ref.view(np.uint64 if dt == np.float64 else np.uint32))
    if layout in ("sub", "gen"):
        # entries of the parent outside the view are untouched
        mask = np.ones(parent.shape, bool)
        if layout == "sub":
            mask[5:5 + m, 2:2 + n] = False
        else:
            mask[::2, :] = False
        assert np.array_equal(parent[mask], before[mask])


def test_mixed_memory_and_pinned(gpu):
    """A on the device, B in pinned host memory, C in pageable host memory."""
    import torch
    rng = np.random.default_rng(5)
    m, n, k = 1024, 2048, 777
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    Bh = rng.uniform(-1, 1, (n, k)).T  # row-major k x n view
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    for prec in (mg.PREC_PLAIN, mg.PREC_OZAKI):
        ref = gu.gemm_device(gpu, A, Bh, C0, 1.0, 1.0, precision=prec)
        ta, ars, acs = gu.to_device(A)
        pinned = torch.empty((n, k), dtype=torch.float64).pin_memory()
        pinned.copy_(torch.from_numpy(np.ascontiguousarray(Bh.T)))
        Bp = pinned.numpy().T
        C = C0.copy(order="F")
        d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 1.0, (ta.data_ptr(), ars, acs),
                         (Bp.ctypes.data, Bp.strides[0] // 8, Bp.strides[1] // 8), (C.ctypes.data, 1, m),
                         precision=prec)
        mg.check(gpu.momms_gemm(ctypes.byref(d), None), gpu)
        assert np.array_equal(C.view(np.uint64), ref.view(np.uint64)), prec


def test_staged_calls_back_to_back(gpu):
    """Consecutive host-staged calls reuse the copy stream; each returns with
    its own C complete."""
    rng = np.random.default_rng(9)
    outs, refs = [], []
    for i in range(6):
        m, n, k = 200 + 37 * i, 640 - 41 * i, 150 + 13 * i
        A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
        B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
        C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
        prec = mg.PREC_OZAKI if i % 2 else mg.PREC_PLAIN
        refs.append(gu.gemm_device(gpu, A, B, C0, 1.0, 0.5, precision=prec))
        C = C0.copy(order="F")
        gu.gemm_host(gpu, A, B, C, 1.0, 0.5, precision=prec)
        outs.append(C)
    for C, R in zip(outs, refs):
        assert np.array_equal(C.view(np.uint64), R.view(np.uint64))
