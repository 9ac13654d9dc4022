"""Block planning of out-of-core (host-resident) calls, without a GPU:
momms_stream_plan with an explicit budget is pure host logic."""
import ctypes

import pytest

import momms_gb300 as mg
from tests import gpu_util as gu


@pytest.fixture(scope="module")
def lib():
    import os
    if not os.path.exists(mg.LIB_PATH):
        from momms_gb300 import build as b
        b.build()
    return mg.load_library()


def _plan(lib, m, n, k, budget, dtype=mg.DTYPE_F64, prec=mg.PREC_PLAIN, mem=mg.MEM_HOST, beta=1.0, mems=None):
    d = gu.make_desc(dtype, m, n, k, 1.0, beta, (1, 1, m), (1, 1, k), (1, 1, m), precision=prec, mem=mem)
    if mems:
        d.a.mem, d.b.mem, d.c.mem = mems
    mb, nb, kb = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    rc = lib.momms_stream_plan(ctypes.byref(d), budget, ctypes.byref(mb), ctypes.byref(nb), ctypes.byref(kb))
    return rc, (mb.value, nb.value, kb.value)


GiB = 1 << 30
MiB = 1 << 20


def _slot(r, c, es):
    up = lambda x: (x + 15) // 16 * 16
    return up(r) * up(c) * es


def test_fits_unblocked(lib):
    rc, p = _plan(lib, 8192, 8192, 8192, 64 * GiB)
    assert rc == mg.OK and p == (8192, 8192, 8192)


@pytest.mark.parametrize("budget_mib", [1024, 512, 300, 160])
def test_blocks_fit_budget(lib, budget_mib):
    m = n = k = 16384
    rc, (mb, nb, kb) = _plan(lib, m, n, k, budget_mib * MiB)
    assert rc == mg.OK
    assert (mb, nb, kb) != (m, n, k)
    for b, full in ((mb, m), (nb, n), (kb, k)):
        assert 0 < b <= full and (b == full or b % 256 == 0)
    # two slots per host operand plus the plain path's work space fit
    used = 2 * (_slot(mb, kb, 8) + _slot(kb, nb, 8) + _slot(mb, nb, 8)) + 21 * MiB + 64 * MiB
    assert used <= budget_mib * MiB


def test_smaller_budget_never_larger_blocks(lib):
    prev = None
    for budget in (4 * GiB, 2 * GiB, GiB, 512 * MiB, 256 * MiB):
        rc, (mb, nb, kb) = _plan(lib, 20000, 12000, 30000, budget)
        assert rc == mg.OK
        area = mb * nb * kb
        if prev is not None:
            assert area <= prev
        prev = area


def test_device_operands_need_no_slots(lib):
    # the same budget allows larger blocks when A and B already live on the device
    budget = 700 * MiB
    _, host_all = _plan(lib, 16384, 16384, 16384, budget)
    _, dev_ab = _plan(lib, 16384, 16384, 16384, budget, mems=(mg.MEM_DEVICE, mg.MEM_DEVICE, mg.MEM_HOST))
    assert dev_ab[0] * dev_ab[1] * dev_ab[2] >= host_all[0] * host_all[1] * host_all[2]


def test_ozaki_slabs_respect_launch_k(lib):
    # one emulated launch sums at most 2^16 products in int32: a plan for a
    # host call with k beyond that uses k slabs, even with room to spare
    rc, (mb, nb, kb) = _plan(lib, 4096, 4096, 100000, 8 * GiB, prec=mg.PREC_OZAKI)
    assert rc == mg.OK and kb <= 65536
    # plain f64 has no such limit and keeps k whole when it fits
    rc, p = _plan(lib, 4096, 4096, 100000, 64 * GiB)
    assert rc == mg.OK and p == (4096, 4096, 100000)


def test_too_small_budget_is_out_of_memory(lib):
    rc, _ = _plan(lib, 16384, 16384, 16384, 8 * MiB)
    assert rc == mg.ERR_OUT_OF_MEMORY
