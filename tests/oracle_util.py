"""ctypes wrappers of the CPU oracle (oracle/goto.c) for the tests.

Test infrastructure: the oracle is the checker, never the thing under test.
"""
import ctypes
import os
import platform

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")

_lib = None
_ref = None
P = ctypes.c_void_p
I64 = ctypes.c_int64


def load():
    global _lib
    if _lib is None:
        import sys
        sys.path.insert(0, ORACLE_DIR)
        import build as oracle_build  # oracle/build.py
        sys.path.pop(0)
        path = oracle_build.build_oracle()
        lib = ctypes.CDLL(path)
        for name, ct in (("oracle_goto_dgemm", ctypes.c_double), ("oracle_goto_sgemm", ctypes.c_float)):
            f = getattr(lib, name)
            f.argtypes = [I64, I64, I64, ct, P, I64, I64, P, I64, I64, ct, P, I64, I64, ctypes.c_int, P]
            f.restype = ctypes.c_int
        lib.oracle_dd_dgemm.argtypes = [I64, I64, I64, ctypes.c_double, P, I64, I64, P, I64, I64, ctypes.c_double,
                                        P, I64, I64, P, P, I64, I64, ctypes.c_int]
        lib.oracle_dd_dgemm.restype = ctypes.c_int
        lib.oracle_dd_dgemm_entries.argtypes = [I64, I64, I64, ctypes.c_double, P, I64, I64, P, I64, I64,
                                                ctypes.c_double, P, I64, I64, P, P, I64, P, P, ctypes.c_int]
        lib.oracle_dd_dgemm_entries.restype = ctypes.c_int
        lib.oracle_freivalds_d.argtypes = [I64, I64, I64, P, I64, I64, P, I64, I64, P, I64, I64, P]
        lib.oracle_freivalds_d.restype = ctypes.c_double
        for name, ct in (("oracle_ukr_d6x8", ctypes.c_double), ("oracle_ukr_s6x16", ctypes.c_float)):
            f = getattr(lib, name)
            f.argtypes = [I64, P, P, P, P, P, I64, I64, P, P]
            f.restype = None
        _lib = lib
    return _lib


def load_ref():
    """The reference's own asm microkernels (x86-64 hosts with the reference
    checkout only); None elsewhere."""
    global _ref
    if _ref is None:
        if platform.machine() not in ("x86_64", "AMD64"):
            return None
        import sys
        sys.path.insert(0, ORACLE_DIR)
        import build as oracle_build
        sys.path.pop(0)
        path = oracle_build.build_ref()
        if path is None:
            return None
        _ref = ctypes.CDLL(path)
    return _ref


def ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def strides(a):
    """(rs, cs) of a 2-D numpy array in elements."""
    return a.strides[0] // a.itemsize, a.strides[1] // a.itemsize


def nthreads():
    return max(1, min(os.cpu_count() or 1, 16))


def goto_gemm(A, B, C, alpha=1.0, beta=1.0, threads=None, ukr=None):
    """C := beta*C + alpha*A*B in place with the reference's Goto algorithm."""
    lib = load()
    m, k = A.shape
    n = B.shape[1]
    f = lib.oracle_goto_dgemm if A.dtype == np.float64 else lib.oracle_goto_sgemm
    ct = ctypes.c_double if A.dtype == np.float64 else ctypes.c_float
    rc = f(m, n, k, ct(alpha), ptr(A), *strides(A), ptr(B), *strides(B), ct(beta), ptr(C), *strides(C),
           threads or nthreads(), ukr)
    assert rc == 0, rc
    return C


def dd_gemm(A, B, C0=None, alpha=1.0, beta=1.0, threads=None):
    """(beta*C0 + alpha*A*B in double-double rounded to f64, |alpha||A||B| + |beta||C0|)."""
    lib = load()
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    m, k = A.shape
    n = B.shape[1]
    out = np.empty((m, n), order="F")
    mag = np.empty((m, n), order="F")
    if C0 is not None:
        C0 = np.asarray(C0, dtype=np.float64)
        c_args = (ptr(C0), *strides(C0))
    else:
        c_args = (None, 0, 0)
    rc = lib.oracle_dd_dgemm(m, n, k, alpha, ptr(A), *strides(A), ptr(B), *strides(B), beta, *c_args,
                             ptr(out), ptr(mag), 1, m, threads or nthreads())
    assert rc == 0
    return out, mag


def dd_gemm_entries(A, B, C0, ii, jj, alpha=1.0, beta=1.0, threads=None):
    """dd_gemm restricted to entries (ii[e], jj[e])."""
    lib = load()
    m, k = A.shape
    n = B.shape[1]
    ii = np.ascontiguousarray(ii, dtype=np.int64)
    jj = np.ascontiguousarray(jj, dtype=np.int64)
    out = np.empty(len(ii))
    mag = np.empty(len(ii))
    if C0 is not None:
        c_args = (ptr(C0), *strides(C0))
    else:
        c_args = (None, 0, 0)
    rc = lib.oracle_dd_dgemm_entries(m, n, k, alpha, ptr(A), *strides(A), ptr(B), *strides(B), beta, *c_args,
                                     ptr(ii), ptr(jj), len(ii), ptr(out), ptr(mag), threads or nthreads())
    assert rc == 0
    return out, mag


def freivalds(A, B, C, w):
    """The reference's residual ||C w - A (B w)||_F^2 (src/util.rs:55-85)."""
    lib = load()
    m, k = A.shape
    n = B.shape[1]
    w = np.ascontiguousarray(w, dtype=np.float64)
    return lib.oracle_freivalds_d(m, n, k, ptr(A), *strides(A), ptr(B), *strides(B), ptr(C), *strides(C), ptr(w))


def bound_ratio(C, Cref, mag, k, u):
    """max_ij |C - Cref| / (2 (k+2) u mag): <= 1 means inside the componentwise
    bound |dC| <= 2k u (|alpha||A||B| + |beta||C0|) (two extra roundings for
    the alpha scale and the beta update)."""
    tol = 2.0 * (k + 2) * u * mag
    err = np.abs(np.asarray(C, dtype=np.float64) - Cref)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(tol > 0, err / np.where(tol > 0, tol, 1.0), np.where(err > 0, np.inf, 0.0))
    return float(r.max()) if r.size else 0.0


def rel_err(C, Cref, mag):
    """max_ij |C - Cref| / mag_ij (the componentwise error the results report)."""
    err = np.abs(np.asarray(C, dtype=np.float64) - Cref)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(mag > 0, err / np.where(mag > 0, mag, 1.0), np.where(err > 0, np.inf, 0.0))
    return float(r.max()) if r.size else 0.0
