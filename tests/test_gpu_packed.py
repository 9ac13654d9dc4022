"""Packed operands (momms_pack): an operand converted once into the form the
kernels read. Every call with packed operands must give the same bits as the
same call on the plain device operands (Ozaki: with the pack's slice count),
in single calls, captured CUDA graphs, grouped plans and the server; misuse
is refused before anything runs."""
import ctypes

import numpy as np
import pytest

import momms_gb300 as mg
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

MODES = [(np.float64, mg.PREC_PLAIN, 0), (np.float64, mg.PREC_OZAKI, 8), (np.float64, mg.PREC_OZAKI, 5),
         (np.float32, mg.PREC_PLAIN, 0), (np.float32, mg.PREC_SPLIT_TF32, 0)]


def _pack(lib, X, prec, role, slices=0, host=False):
    dt = mg.DTYPE_F64 if X.dtype == np.float64 else mg.DTYPE_F32
    rows, cols = X.shape
    keep = None
    if host:
        op = mg.Operand(X.ctypes.data, X.strides[0] // X.itemsize, X.strides[1] // X.itemsize, mg.MEM_HOST, 0)
    else:
        t, rs, cs = gu.to_device(X)
        keep = t
        op = mg.Operand(t.data_ptr(), rs, cs, mg.MEM_DEVICE, 0)
    h = ctypes.c_void_p()
    mg.check(lib.momms_pack(dt, prec, role, rows, cols, ctypes.byref(op), slices, None, ctypes.byref(h)), lib)
    del keep
    return h


def _call(lib, A, B, C0, prec, pa=None, pb=None, slices=0, alpha=1.0, beta=0.5, stream=None):
    """momms_gemm on device copies; pa / pb replace A / B by packs."""
    import torch
    dt = mg.DTYPE_F64 if C0.dtype == np.float64 else mg.DTYPE_F32
    m, k = A.shape
    n = B.shape[1]
    ta, ars, acs = gu.to_device(A)
    tb, brs, bcs = gu.to_device(B)
    tc, crs, ccs = gu.to_device(C0)
    d = gu.make_desc(dt, m, n, k, alpha, beta, (ta.data_ptr(), ars, acs), (tb.data_ptr(), brs, bcs),
                     (tc.data_ptr(), crs, ccs), precision=prec, slices=slices)
    if pa is not None:
        d.a = mg.Operand(pa.value, 0, 0, mg.MEM_PACKED, 0)
    if pb is not None:
        d.b = mg.Operand(pb.value, 0, 0, mg.MEM_PACKED, 0)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    rc = lib.momms_gemm(ctypes.byref(d), ctypes.c_void_p(s))
    torch.cuda.synchronize()
    return rc, tc.cpu().numpy()


def _bits(x):
    return x.view(np.uint64 if x.dtype == np.float64 else np.uint32)


@pytest.mark.parametrize("mode", MODES, ids=["f64", "ozaki8", "ozaki5", "f32", "tf32"])
def test_packed_bitwise(gpu, mode):
    dt, prec, slices = mode
    rng = np.random.default_rng(slices + prec * 7)
    m, n, k = 300, 517, 260
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)).astype(dt))
    B = np.ascontiguousarray(rng.uniform(-1, 1, (k, n)).astype(dt))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)).astype(dt))
    ns = slices if prec == mg.PREC_OZAKI else 0
    rc, ref = _call(gpu, A, B, C0, prec, slices=ns)
    assert rc == mg.OK
    pa = _pack(gpu, A, prec, mg.ROLE_A, slices, host=True)
    pb = _pack(gpu, B, prec, mg.ROLE_B, slices)
    try:
        assert gpu.momms_packed_bytes(pa) > 0
        for use in ((pa, None), (None, pb), (pa, pb)):
            # desc.slices 0: the pack's count is used
            rc, got = _call(gpu, A, B, C0, prec, pa=use[0], pb=use[1])
            assert rc == mg.OK, gpu.momms_last_error()
            assert np.array_equal(_bits(got), _bits(ref)), use
    finally:
        gpu.momms_packed_destroy(pa)
        gpu.momms_packed_destroy(pb)


def test_packed_misuse_is_refused(gpu):
    rng = np.random.default_rng(1)
    m, n, k = 64, 48, 40
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.zeros((m, n), order="F")
    pa7 = _pack(gpu, A, mg.PREC_OZAKI, mg.ROLE_A, 7)
    pb8 = _pack(gpu, B, mg.PREC_OZAKI, mg.ROLE_B, 8)
    pa_plain = _pack(gpu, A, mg.PREC_PLAIN, mg.ROLE_A)
    try:
        cases = [
            dict(prec=mg.PREC_OZAKI, pa=pa7, pb=pb8),             # slice counts differ
            dict(prec=mg.PREC_OZAKI, pa=pa7, slices=8),            # desc asks for another count
            dict(prec=mg.PREC_PLAIN, pa=pa7),                      # pack made for another precision
            dict(prec=mg.PREC_OZAKI, pb=pa7),                      # A's pack in B's place
        ]
        for c in cases:
            rc, _ = _call(gpu, A, B, C0, c["prec"], pa=c.get("pa"), pb=c.get("pb"), slices=c.get("slices", 0))
            assert rc == mg.ERR_INVALID_ARG, c
        # sizes must match the call
        rc, _ = _call(gpu, A[:, :20].copy(order="F"), B[:20, :].copy(order="F"), C0, mg.PREC_PLAIN, pa=pa_plain)
        assert rc == mg.ERR_INVALID_ARG
        # C cannot be packed
        d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 0.0, (1, 1, m), (1, 1, k), (pa_plain.value, 0, 0))
        d.c.mem = mg.MEM_PACKED
        assert gpu.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
        # the pack's source may not be a pack, sizes must be positive
        h = ctypes.c_void_p()
        op = mg.Operand(pa_plain.value, 0, 0, mg.MEM_PACKED, 0)
        assert gpu.momms_pack(mg.DTYPE_F64, mg.PREC_PLAIN, mg.ROLE_A, m, k, ctypes.byref(op), 0, None,
                              ctypes.byref(h)) == mg.ERR_INVALID_ARG
    finally:
        for h in (pa7, pb8, pa_plain):
            assert gpu.momms_packed_destroy(h) == mg.OK
    # a destroyed pack is refused
    rc, _ = _call(gpu, A, B, C0, mg.PREC_PLAIN, pa=pa_plain)
    assert rc == mg.ERR_INVALID_ARG


def test_packed_ozaki_call_captures_in_a_graph(gpu):
    """With both operands packed the emulated call needs no host round trip:
    it captures into a CUDA graph and the replays give the same bits."""
    import torch
    rng = np.random.default_rng(3)
    m, n, k = 512, 384, 640
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    B = np.asfortranarray(rng.uniform(-1, 1, (k, n)))
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    rc, ref = _call(gpu, A, B, C0, mg.PREC_OZAKI, slices=8, beta=0.0)
    assert rc == mg.OK
    pa = _pack(gpu, A, mg.PREC_OZAKI, mg.ROLE_A, 8)
    pb = _pack(gpu, B, mg.PREC_OZAKI, mg.ROLE_B, 8)
    try:
        tc = torch.zeros((n, m), dtype=torch.float64, device="cuda").t()
        d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 0.0, (pa.value, 0, 0), (pb.value, 0, 0),
                         (tc.data_ptr(), 1, m), precision=mg.PREC_OZAKI)
        d.a.mem = mg.MEM_PACKED
        d.b.mem = mg.MEM_PACKED
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):  # warm-up outside the capture
            mg.check(gpu.momms_gemm(ctypes.byref(d), ctypes.c_void_p(s.cuda_stream)), gpu)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            mg.check(gpu.momms_gemm(ctypes.byref(d), ctypes.c_void_p(s.cuda_stream)), gpu)
        for _ in range(3):
            tc.zero_()
            g.replay()
            torch.cuda.synchronize()
            assert np.array_equal(_bits(tc.cpu().numpy()), _bits(ref))
        del g
    finally:
        gpu.momms_packed_destroy(pa)
        gpu.momms_packed_destroy(pb)


def test_packed_in_plans_and_server(gpu):
    import torch
    rng = np.random.default_rng(4)
    m, n, k = 200, 300, 250
    A = np.asfortranarray(rng.uniform(-1, 1, (m, k)))
    Bs = [np.asfortranarray(rng.uniform(-1, 1, (k, n))) for _ in range(3)]
    C0 = np.asfortranarray(rng.uniform(-1, 1, (m, n)))
    pa_plain = _pack(gpu, A, mg.PREC_PLAIN, mg.ROLE_A)
    pa_oz = _pack(gpu, A, mg.PREC_OZAKI, mg.ROLE_A, 8)
    try:
        refs, descs, keep = [], (mg.GemmDesc * 4)(), []
        plan_items = [(mg.PREC_PLAIN, pa_plain, Bs[0]), (mg.PREC_OZAKI, pa_oz, Bs[1]), (mg.PREC_PLAIN, pa_plain, Bs[2]),
                      (mg.PREC_OZAKI, pa_oz, Bs[0])]
        for i, (prec, pa, B) in enumerate(plan_items):
            rc, r = _call(gpu, A, B, C0, prec, slices=8 if prec == mg.PREC_OZAKI else 0)
            assert rc == mg.OK
            refs.append(r)
            tb, brs, bcs = gu.to_device(B)
            tc, crs, ccs = gu.to_device(C0)
            keep.append((tb, tc))
            d = gu.make_desc(mg.DTYPE_F64, m, n, k, 1.0, 0.5, (pa.value, 0, 0), (tb.data_ptr(), brs, bcs),
                             (tc.data_ptr(), crs, ccs), precision=prec)
            d.a.mem = mg.MEM_PACKED
            descs[i] = d
        s = torch.cuda.current_stream().cuda_stream
        mg.check(gpu.momms_gemm_grouped(descs, 4, ctypes.c_void_p(s)), gpu)
        torch.cuda.synchronize()
        for (tb, tc), r in zip(keep, refs):
            assert np.array_equal(_bits(tc.cpu().numpy()), _bits(r))
        # the server takes the same requests
        for tb, tc in keep:
            tc.copy_(torch.from_numpy(C0).cuda())
        cfg = mg.ServerConfig(hbm_budget_bytes=8 << 30, max_batch=4, max_inflight=2, queue_capacity=64)
        srv = ctypes.c_void_p()
        mg.check(gpu.momms_server_create(ctypes.byref(cfg), ctypes.byref(srv)), gpu)
        try:
            for i in range(4):
                rid = ctypes.c_uint64()
                mg.check(gpu.momms_server_submit(srv, ctypes.byref(descs[i]), ctypes.byref(rid)), gpu)
            mg.check(gpu.momms_server_drain(srv, 60.0), gpu)
        finally:
            gpu.momms_server_destroy(srv)
        for (tb, tc), r in zip(keep, refs):
            assert np.array_equal(_bits(tc.cpu().numpy()), _bits(r))
    finally:
        gpu.momms_packed_destroy(pa_plain)
        gpu.momms_packed_destroy(pa_oz)
