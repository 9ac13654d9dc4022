"""Launch configurations and the autotuner.

A plain problem's configuration is an output tile (f32: 128 x 128 or 64 x 64)
and a k-split count, from the tuning table (keyed by shape bucket) or the
model. Within a split every output is the same fma chain over k, so the tile
never changes a result; and the configuration depends on the problem's shape
alone, so a problem gives the same bits alone and in any batch, tuned or not.
"""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clean_table(gpu):
    gpu.momms_tune_clear()
    yield
    gpu.momms_tune_clear()


def _mats(rng, m, n, k, dt, orders="FFF"):
    def mk(r, c, o):
        x = rng.uniform(-1, 1, (r, c)).astype(dt)
        return np.asfortranarray(x) if o == "F" else np.ascontiguousarray(x)
    return mk(m, k, orders[0]), mk(k, n, orders[1]), mk(m, n, orders[2])


@pytest.mark.parametrize("shape,orders", [((300, 200, 700), "FFF"), ((129, 65, 2000), "CFC"), ((64, 64, 64), "FCF"),
                                          ((1000, 777, 300), "FFF")])
def test_f32_tiles_give_the_same_bits(gpu, shape, orders):
    m, n, k = shape
    rng = np.random.default_rng(m + n + k)
    A, B, C0 = _mats(rng, m, n, k, np.float32, orders)
    results = []
    for tile in (0, 1):
        gpu.momms_tune_clear()
        mg.check(gpu.momms_tune_import(f"1 0 {m} {n} {k} 1 {tile}".encode()), gpu)
        results.append(gu.gemm_device(gpu, A, B, C0, 0.75, -0.5))
    assert np.array_equal(results[0], results[1])
    ref, mag = ou.dd_gemm(A, B, C0, 0.75, -0.5)
    assert ou.bound_ratio(results[1], ref, mag, k, 2.0**-24) <= 1.0


def test_small_tile_with_split_k(gpu):
    """The 64 x 64 tile with a split count from the table: inside the FP32
    bound, and the same bits on every run (fixed reduction order)."""
    m, n, k = 200, 180, 9000
    rng = np.random.default_rng(4)
    A, B, C0 = _mats(rng, m, n, k, np.float32)
    mg.check(gpu.momms_tune_import(f"1 0 {m} {n} {k} 6 1".encode()), gpu)
    C1 = gu.gemm_device(gpu, A, B, C0)
    C2 = gu.gemm_device(gpu, A, B, C0)
    assert np.array_equal(C1, C2)
    ref, mag = ou.dd_gemm(A, B, C0)
    assert ou.bound_ratio(C1, ref, mag, k, 2.0**-24) <= 1.0


def _batch(rng, count):
    descs, keep = [], []
    for i in range(count):
        dt = np.float64 if i % 2 == 0 else np.float32
        m, n, k = (int(x) for x in np.exp(rng.uniform(np.log(32), np.log(600), 3)))
        A, B, C0 = _mats(rng, m, n, k, dt)
        ta, _, _ = gu.to_device(A)
        tb, _, _ = gu.to_device(B)
        tc, _, _ = gu.to_device(C0)
        keep.append((A, B, C0, tc))
        descs.append(gu.make_desc(mg.DTYPE_F64 if dt == np.float64 else mg.DTYPE_F32, m, n, k, 1.0, 1.0,
                                  (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, k), (tc.data_ptr(), 1, m),
                                  mem=mg.MEM_DEVICE))
        keep[-1] = keep[-1] + (ta, tb)
    return (mg.GemmDesc * count)(*descs), keep


def test_autotune_batch_then_grouped_equals_single(gpu):
    import torch
    rng = np.random.default_rng(77)
    arr, keep = _batch(rng, 24)
    tuned = ctypes.c_int32(0)
    mg.check(gpu.momms_autotune_batch(arr, len(arr), None, ctypes.byref(tuned)), gpu)
    assert tuned.value >= 2
    need = ctypes.c_size_t(0)
    mg.check(gpu.momms_tune_export(None, 0, ctypes.byref(need)), gpu)
    buf = ctypes.create_string_buffer(need.value)
    mg.check(gpu.momms_tune_export(buf, need.value, None), gpu)
    lines = buf.value.decode().strip().split("\n")
    assert len(lines) == tuned.value
    # the tuner wrote only scratch: every C still holds its input
    for A, B, C0, tc, ta, tb in keep:
        assert np.array_equal(tc.cpu().numpy(), C0)
    mg.check(gpu.momms_gemm_grouped(arr, len(arr), None), gpu)
    torch.cuda.synchronize()
    for A, B, C0, tc, ta, tb in keep:
        alone = gu.gemm_device(gpu, A, B, C0)
        assert np.array_equal(tc.cpu().numpy(), alone)


def test_autotune_reports_its_choice(gpu):
    m, n, k = 256, 256, 4096
    rng = np.random.default_rng(9)
    A, B, C0 = _mats(rng, m, n, k, np.float32)
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F32, m, n, k, 1.0, 1.0, (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, k),
                     (tc.data_ptr(), 1, m), mem=mg.MEM_DEVICE)
    res = mg.TuneResult()
    mg.check(gpu.momms_autotune(ctypes.byref(d), ctypes.byref(res), None), gpu)
    assert res.tile in (0, 1) and res.splits >= 1 and res.candidates > 10 and res.best_ms > 0
