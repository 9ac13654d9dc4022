"""Helpers for the GPU tests: move numpy operands to the device with their
strides intact and call the library through its C ABI."""
import ctypes

import numpy as np

import momms_gb300 as mg


def to_device(x):
    """numpy 2-D array (any positive strides) -> CUDA tensor with the same
    element strides. Returns (tensor, rs, cs)."""
    import torch
    rs, cs = x.strides[0] // x.itemsize, x.strides[1] // x.itemsize
    rows, cols = x.shape
    span = (rows - 1) * rs + (cols - 1) * cs + 1 if rows and cols else 1
    flat = np.lib.stride_tricks.as_strided(x, shape=(span,), strides=(x.itemsize,)) if rows and cols else \
        np.zeros(1, x.dtype)
    # copy the whole spanned storage so that the same strides address the same elements
    base = torch.from_numpy(np.array(flat)).cuda()
    t = torch.as_strided(base, (rows, cols), (rs, cs))
    return t, rs, cs


def from_device(t, like):
    return t.cpu().numpy().astype(like.dtype, copy=False)


def make_desc(dtype, m, n, k, alpha, beta, a, b, c, precision=mg.PREC_PLAIN, mem=mg.MEM_AUTO,
              target_rel_err=0.0, slices=0):
    """a, b, c: (ptr, rs, cs) triples."""
    d = mg.GemmDesc()
    d.dtype = dtype
    d.precision = precision
    d.m, d.n, d.k = m, n, k
    d.alpha, d.beta = alpha, beta
    d.a = mg.Operand(a[0], a[1], a[2], mem, 0)
    d.b = mg.Operand(b[0], b[1], b[2], mem, 0)
    d.c = mg.Operand(c[0], c[1], c[2], mem, 0)
    d.target_rel_err = target_rel_err
    d.slices = slices
    d.flags = 0
    return d


def gemm_device(lib, A, B, C0, alpha=1.0, beta=1.0, precision=mg.PREC_PLAIN, stream=None, **kw):
    """Runs C := beta*C0 + alpha*A*B on device copies of the operands and
    returns the result as a numpy array with C0's layout."""
    import torch
    dt = mg.DTYPE_F64 if A.dtype == np.float64 else mg.DTYPE_F32
    m, k = A.shape
    n = B.shape[1]
    ta, ars, acs = to_device(A)
    tb, brs, bcs = to_device(B)
    tc, crs, ccs = to_device(C0)
    d = make_desc(dt, m, n, k, alpha, beta, (ta.data_ptr(), ars, acs), (tb.data_ptr(), brs, bcs),
                  (tc.data_ptr(), crs, ccs), precision=precision, **kw)
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    mg.check(lib.momms_gemm(ctypes.byref(d), ctypes.c_void_p(s)), lib)
    torch.cuda.synchronize()
    out = np.empty_like(C0)
    out[...] = tc.cpu().numpy()
    return out


def gemm_host(lib, A, B, C, alpha=1.0, beta=1.0, precision=mg.PREC_PLAIN, **kw):
    """Runs the call with host (numpy) operands; C is updated in place."""
    dt = mg.DTYPE_F64 if A.dtype == np.float64 else mg.DTYPE_F32
    m, k = A.shape
    n = B.shape[1]

    def trip(x):
        return (x.ctypes.data, x.strides[0] // x.itemsize, x.strides[1] // x.itemsize)

    d = make_desc(dt, m, n, k, alpha, beta, trip(A), trip(B), trip(C), precision=precision, mem=mg.MEM_HOST, **kw)
    mg.check(lib.momms_gemm(ctypes.byref(d), None), lib)
    return C
