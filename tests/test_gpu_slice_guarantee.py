"""The automatic slice count holds for every entry, or the call says it cannot.

An emulated FP64 call with slices == 0 chooses its slice count from the
requested componentwise error. The choice rests on a rigorous bound evaluated
over every entry of C (a bf16 magnitude product on the tensor cores), not on
a sample: the tests below build entries a sample misses and check that the
result meets the target on every entry against the double-double oracle, that
momms_last_info's bound_rel_err is a true bound, and that a target no slice
count can guarantee returns MOMMS_ERR_TARGET_UNREACHABLE with the 15-slice
result in C.
"""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu
from tests import oracle_util as ou

pytestmark = pytest.mark.gpu

U64 = 2.0**-53
MASK = (1 << 64) - 1


def sampled_rows(m, n, row_blocks=8, cols=8):
    """Rows the sampled estimate looks at (the library's sample positions)."""
    rows = set()
    for y in range(cols):
        for x in range(row_blocks):
            h = (0x9E3779B97F4A7C15 * (x * 131 + y * 7 + 1)) & MASK
            h ^= h >> 31
            h = (h * 0xBF58476D1CE4E5B9) & MASK
            h ^= h >> 29
            i0 = h % (m - 31) if m > 32 else 0
            rows.update(range(i0, i0 + 32))
    return rows


def adversarial(m, n, k, seed, spread=1e-10):
    """Uniform operands plus one row i* with a 1 : spread in-row range whose
    large entry meets a zero of B's column j*: (|A||B|)_{i*j*} is about
    spread * k / 4 while the digits of row i* are scaled to its entry 1."""
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    missed = sorted(set(range(m)) - sampled_rows(m, n))
    i = missed[len(missed) // 2] if missed else m // 2
    j = n // 3
    A[i, 0] = 1.0
    A[i, 1:] *= spread
    B[0, j] = 0.0
    return A, B, i, j


def _info(gpu):
    info = mg.CallInfo()
    mg.check(gpu.momms_last_info(ctypes.byref(info)), gpu)
    return info


def _run(gpu, A, B, target, host=False, slices=0):
    m, n = A.shape[0], B.shape[1]
    C0 = np.zeros((m, n), order="F")
    if host:
        C = C0.copy(order="F")
        d = gu.make_desc(mg.DTYPE_F64, m, n, A.shape[1], 1.0, 0.0, (A.ctypes.data, 1, m), (B.ctypes.data, 1, A.shape[1]),
                         (C.ctypes.data, 1, m), precision=mg.PREC_OZAKI, mem=mg.MEM_HOST, target_rel_err=target,
                         slices=slices)
        rc = gpu.momms_gemm(ctypes.byref(d), None)
        return rc, C
    import torch
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(C0)
    d = gu.make_desc(mg.DTYPE_F64, m, n, A.shape[1], 1.0, 0.0, (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, A.shape[1]),
                     (tc.data_ptr(), 1, m), precision=mg.PREC_OZAKI, target_rel_err=target, slices=slices)
    rc = gpu.momms_gemm(ctypes.byref(d), None)
    torch.cuda.synchronize()
    return rc, tc.cpu().numpy()


def _errors(C, A, B):
    ref, mag = ou.dd_gemm(A, B, None, beta=0.0)
    err = np.abs(C - ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(mag > 0, err / np.where(mag > 0, mag, 1.0), np.where(err > 0, np.inf, 0.0))
    return rel


@pytest.mark.parametrize("host", [False, True])
def test_adversarial_row_meets_target_on_every_entry(gpu, host):
    target = 1e-14
    # host operands: B and C arrive by column chunks (n >= 1024), the count
    # starts from the sample and is verified before C is written
    m, n, k = (2048, 1100, 400) if host else (600, 520, 500)
    A, B, i, j = adversarial(m, n, k, 17 + host)
    rc, C = _run(gpu, A, B, target, host=host)
    assert rc == mg.OK, gpu.momms_last_error()
    info = _info(gpu)
    rel = _errors(C, A, B)
    assert rel.max() <= target, (rel.max(), np.unravel_index(rel.argmax(), rel.shape), (i, j), info.slices)
    assert 0.0 < info.bound_rel_err <= target
    assert rel.max() <= info.bound_rel_err + 2 * U64  # the bound is a bound (plus C's final rounding)
    # the sampled estimate's count (what a sample-only choice ran) misses entry (i, j)
    rc7, C7 = _run(gpu, A, B, target, host=host, slices=7)
    assert rc7 == mg.OK
    assert _errors(C7, A, B)[i, j] > target
    assert info.slices > 7


def test_uniform_data_keeps_seven_slices_at_fp64_level(gpu):
    """The guarantee costs no extra slice on the benchmark's data."""
    rng = np.random.default_rng(5)
    m, n, k = 1024, 1024, 1024
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    rc, C = _run(gpu, A, B, 0.0)
    assert rc == mg.OK
    info = _info(gpu)
    assert info.slices == 7
    rel = _errors(C, A, B)
    assert rel.max() <= info.bound_rel_err + 2 * U64
    assert info.bound_rel_err <= 2.0**-52


def test_unreachable_target_is_reported_with_the_15_slice_result(gpu):
    rng = np.random.default_rng(6)
    m, n, k = 300, 280, 350
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    rc, C = _run(gpu, A, B, 1e-45)  # beyond 15 slices of 8 bits
    assert rc == mg.ERR_TARGET_UNREACHABLE
    info = _info(gpu)
    assert info.slices == 15
    assert info.bound_rel_err > 1e-45
    assert _errors(C, A, B).max() <= 4 * U64  # C holds the 15-slice result


def test_entries_beyond_fp32_range_are_uncovered(gpu):
    """Every product term of entry (i, j) is below 2^-126 of the row's and
    column's scale: no slice count reaches it, and the call says so."""
    A, B, i, j = adversarial(300, 260, 300, 9, spread=1e-200)
    rc, C = _run(gpu, A, B, 1e-14)
    assert rc == mg.ERR_TARGET_UNREACHABLE
    assert _info(gpu).bound_rel_err == float("inf")


def test_structural_zeros_are_exact_and_covered(gpu):
    """Block-diagonal operands: the off-diagonal blocks of C have no nonzero
    product term. The indicator pass shows they are exact, so the bound holds
    for every entry and the call succeeds."""
    rng = np.random.default_rng(12)
    m, n, k = 320, 288, 256
    A = np.zeros((m, k), order="F")
    B = np.zeros((k, n), order="F")
    A[:160, :128] = rng.uniform(-1, 1, (160, 128))
    A[160:, 128:] = rng.uniform(-1, 1, (160, 128))
    B[:128, :144] = rng.uniform(-1, 1, (128, 144))
    B[128:, 144:] = rng.uniform(-1, 1, (128, 144))
    rc, C = _run(gpu, A, B, 1e-14)
    assert rc == mg.OK, gpu.momms_last_error()
    assert np.all(C[:160, 144:] == 0.0) and np.all(C[160:, :144] == 0.0)
    assert _errors(C, A, B).max() <= 1e-14


def test_plan_choice_is_guaranteed(gpu):
    """A plan chooses an emulated problem's count once at creation, with the
    same guarantee; an unreachable target refuses the plan."""
    import torch
    A, B, i, j = adversarial(600, 520, 500, 23)
    m, k = A.shape
    n = B.shape[1]
    ta, _, _ = gu.to_device(A)
    tb, _, _ = gu.to_device(B)
    tc, _, _ = gu.to_device(np.zeros((m, n), order="F"))
    d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 0.0, (ta.data_ptr(), 1, m), (tb.data_ptr(), 1, k),
                     (tc.data_ptr(), 1, m), precision=mg.PREC_OZAKI, mem=mg.MEM_DEVICE, target_rel_err=1e-14)
    arr = (mg.GemmDesc * 1)(d)
    plan = ctypes.c_void_p()
    mg.check(gpu.momms_plan_create(arr, 1, ctypes.byref(plan)), gpu)
    mg.check(gpu.momms_plan_launch(plan, None), gpu)
    torch.cuda.synchronize()
    mg.check(gpu.momms_plan_destroy(plan), gpu)
    assert _errors(tc.cpu().numpy(), A, B).max() <= 1e-14
    arr[0].target_rel_err = 1e-45
    assert gpu.momms_plan_create(arr, 1, ctypes.byref(plan)) == mg.ERR_TARGET_UNREACHABLE


def test_every_slice_count_up_to_the_most(gpu):
    """Fixed counts 1..15 on data with an exponent spread (phi = 2): the error
    falls with every added slice until only C's FP64 rounding is left, up to
    the largest count (its 120-bit digits need the full 128-bit split)."""
    rng = np.random.default_rng(31)
    m, n, k = 260, 200, 300
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)) * np.exp(2.0 * rng.standard_normal((m, k))))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)) * np.exp(2.0 * rng.standard_normal((k, n))))
    errs = []
    for s in range(1, 16):
        rc, C = _run(gpu, A, B, 0.0, slices=s)
        assert rc == mg.OK, (s, gpu.momms_last_error())
        errs.append(_errors(C, A, B).max())
    for s in range(1, 9):
        assert errs[s] < errs[s - 1] / 16, (s + 1, errs)
    assert max(errs[9:]) <= 2 * U64, errs  # 10 slices and more: FP64 rounding of C only
