"""The measurement helpers of momms_gb300.sweep, without a GPU: the exact
products behind the sampled error, the error itself, and the roofline bound
(min of peak and intensity x HBM)."""
import math

import numpy as np

from momms_gb300 import sweep


def test_two_prod_is_error_free():
    rng = np.random.default_rng(3)
    a = rng.standard_normal(1000) * np.exp(rng.uniform(-30, 30, 1000))
    b = rng.standard_normal(1000) * np.exp(rng.uniform(-30, 30, 1000))
    p, e = sweep._two_prod(a, b)
    for x, y, pp, ee in zip(a[:50], b[:50], p[:50], e[:50]):
        # p + e == x*y exactly: compare with rational arithmetic
        from fractions import Fraction
        assert Fraction(pp) + Fraction(ee) == Fraction(x) * Fraction(y)


def test_sampled_error_orders():
    rng = np.random.default_rng(0)
    A = rng.uniform(-1, 1, (64, 300))
    B = rng.uniform(-1, 1, (300, 48))
    exact_like = sweep.sampled_error(A, B, A @ B)
    assert 0.0 <= exact_like < 1e-15
    f32 = (A.astype(np.float32) @ B.astype(np.float32)).astype(np.float64)
    assert 1e-9 < sweep.sampled_error(A, B, f32) < 1e-6
    bad = A @ B
    bad[5, :] = np.nan
    assert math.isinf(sweep.sampled_error(A, B, bad, samples=2000))


def test_roofline_bound():
    pk = {"hbm_gbs": 6760.6, "f16_tflops": 1891.8, "tf32_tflops": 945.9, "f64_tflops": 1.1, "f32_tflops": 78.0}
    # rank-64 f64: intensity 2*8192*8192*64 / (8*(2*8192*64 + 8192^2)) ~ 15.8 flop/B -> compute-bound at 1.1
    o = sweep.roofline({"dtype": "f64", "prec": "plain", "m": 8192, "n": 8192, "k": 64, "ms": 8.0,
                        "tflops": 1.07}, pk)
    assert abs(o["bound_tflops"] - 1.1) < 1e-12
    # f32 rank-64 (31 flop/B) is still compute-bound; rank-8 (4 flop/B) is HBM-bound below 78
    o = sweep.roofline({"dtype": "f32", "prec": "plain", "m": 8192, "n": 8192, "k": 64, "ms": 0.35,
                        "tflops": 24.5}, pk)
    assert abs(o["bound_tflops"] - 78.0) < 1e-12
    o = sweep.roofline({"dtype": "f32", "prec": "plain", "m": 8192, "n": 8192, "k": 8, "ms": 0.1,
                        "tflops": 10.7}, pk)
    flops, bytes_ = 2.0 * 8192 * 8192 * 8, 4 * (8192 * 8 * 2 + 8192 * 8192)
    assert abs(o["bound_tflops"] - flops / bytes_ * 6760.6 / 1e3) < 1e-9 and o["bound_tflops"] < 78.0
    # emulated FP64 without a pair count: no bound; with 28 slice products per
    # output product the peak is the fp16 rate / 28 (67.6 TFLOP/s), below the
    # rank-64 HBM limit (15.8 flop/B x 6.76 TB/s = 107 TFLOP/s)
    assert "bound_tflops" not in sweep.roofline({"dtype": "f64", "prec": "ozaki", "m": 64, "n": 64, "k": 64,
                                                 "ms": 1.0, "tflops": 1.0}, pk)
    o = sweep.roofline({"dtype": "f64", "prec": "ozaki", "m": 8192, "n": 8192, "k": 64, "ms": 1.17,
                        "tflops": 7.35, "slices": 7, "pairs": 28}, pk)
    assert abs(o["bound_tflops"] - 1891.8 / 28) < 1e-9
    assert abs(o["frac_of_bound"] - 7.35 / (1891.8 / 28)) < 1e-12
    # rank 8: the HBM limit (2 flop/B x 6.76 TB/s) is the bound
    o = sweep.roofline({"dtype": "f64", "prec": "ozaki", "m": 8192, "n": 8192, "k": 8, "ms": 0.5,
                        "tflops": 2.0, "slices": 7, "pairs": 28}, pk)
    flops, bytes_ = 2.0 * 8192 * 8192 * 8, 8 * (8192 * 8 * 2 + 8192 * 8192)
    assert abs(o["bound_tflops"] - flops / bytes_ * 6760.6 / 1e3) < 1e-9


def test_slice_sweep_table_format():
    from tests import slice_sweep
    rows = [{"s": 2048, "phi": 0.5, "slices": "plain", "used": 0, "ms": 18.7, "tflops": 0.92, "err": 1.1e-16,
             "bound": None, "unreachable": False, "entries_checked": 2048 * 2048},
            {"s": 2048, "phi": 8.0, "slices": "auto 1e-14", "used": 15, "ms": 2.0, "tflops": 8.6, "err": 3e-15,
             "bound": 2e-12, "unreachable": True, "entries_checked": 2048 * 2048}]
    t = slice_sweep.table(rows).split("\n")
    assert len(t) == 4 and t[2].startswith("| 2048 | 0.5 | plain | — |")
    assert "(target unreachable)" in t[3]
