"""The C ABI library, checked without a GPU: it loads, exports every function
that include/*.h declares, and rejects bad descriptors before touching the
device."""
import ctypes
import glob
import os
import re

import pytest

import momms_gb300 as mg
from tests import gpu_util as gu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(mg.LIB_PATH):
        from momms_gb300 import build as b
        b.build()
    return mg.load_library()


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(momms_\w+)\s*\(", text)
    return sorted(set(names))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 8
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version(lib):
    assert lib.momms_abi_version() == 2


def test_status_strings(lib):
    for code in range(0, 11):
        s = lib.momms_status_string(code).decode()
        assert s and s != "unknown status"
    assert lib.momms_status_string(12345).decode() == "unknown status"


def _desc(**kw):
    d = gu.make_desc(mg.DTYPE_F64, 4, 5, 6, 1.0, 1.0, (8, 1, 4), (8, 1, 6), (8, 1, 4))
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_validate_accepts_good_desc(lib):
    assert lib.momms_gemm_validate(ctypes.byref(_desc())) == mg.OK


@pytest.mark.parametrize("field,value,code", [
    ("m", -1, mg.ERR_INVALID_ARG),
    ("k", -5, mg.ERR_INVALID_ARG),
    ("dtype", 7, mg.ERR_INVALID_ARG),
    ("precision", 9, mg.ERR_INVALID_ARG),
    ("flags", 1, mg.ERR_INVALID_ARG),
    ("m", 2**31, mg.ERR_INVALID_ARG),
])
def test_validate_rejects(lib, field, value, code):
    assert lib.momms_gemm_validate(ctypes.byref(_desc(**{field: value}))) == code


def test_validate_rejects_null_and_bad_strides(lib):
    d = _desc()
    d.a = mg.Operand(None, 1, 4, 0, 0)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
    d = _desc()
    d.c = mg.Operand(8, 3, 3, 0, 0)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
    d = _desc()
    d.b = mg.Operand(8, -1, 6, 0, 0)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
    d = _desc()
    d.a = mg.Operand(8, 1, 4, 5, 0)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
    assert lib.momms_gemm_validate(None) == mg.ERR_INVALID_ARG


def test_validate_mode_dtype_pairs(lib):
    d = _desc(dtype=mg.DTYPE_F32, precision=mg.PREC_OZAKI)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_UNSUPPORTED
    d = _desc(dtype=mg.DTYPE_F64, precision=mg.PREC_SPLIT_TF32)
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_UNSUPPORTED


def test_last_error_message(lib):
    lib.momms_gemm_validate(ctypes.byref(_desc(m=-1)))
    assert b"negative" in lib.momms_last_error()


def test_tune_table_text_roundtrip(lib):
    lib.momms_tune_clear()
    # entries are keyed by shape bucket (ceil(log2) of m, n, k) and exported
    # as the bucket's largest shape; the tile field is optional on import
    assert lib.momms_tune_import(b"0 0 100 200 300 4\n1 0 64 64 9000 8 1\n") == mg.OK
    need = ctypes.c_size_t(0)
    assert lib.momms_tune_export(None, 0, ctypes.byref(need)) == mg.OK
    buf = ctypes.create_string_buffer(need.value)
    assert lib.momms_tune_export(buf, need.value, None) == mg.OK
    rows = sorted(buf.value.decode().strip().split("\n"))
    assert rows == ["0 0 128 256 512 4 0", "1 0 64 64 16384 8 1"]
    # a shape of the same bucket replaces the entry
    assert lib.momms_tune_import(b"0 0 120 129 260 6") == mg.OK
    assert lib.momms_tune_export(None, 0, ctypes.byref(need)) == mg.OK
    buf = ctypes.create_string_buffer(need.value)
    assert lib.momms_tune_export(buf, need.value, None) == mg.OK
    assert "0 0 128 256 512 6 0" in buf.value.decode()
    assert lib.momms_tune_import(b"0 0 8 8 8 4 1") == mg.ERR_INVALID_ARG  # f64 has one tile
    small = ctypes.create_string_buffer(4)
    assert lib.momms_tune_export(small, 4, None) == mg.ERR_INVALID_ARG
    assert lib.momms_tune_import(b"garbage") == mg.ERR_INVALID_ARG
    assert lib.momms_tune_import(b"0 0 1 1 1 99") == mg.ERR_INVALID_ARG
    lib.momms_tune_clear()
    assert lib.momms_tune_export(None, 0, ctypes.byref(need)) == mg.OK and need.value == 1


def test_packed_operand_handles_checked_without_a_gpu(lib):
    """A MOMMS_MEM_PACKED operand must be a live pack: a foreign pointer is
    refused by validation (looked up, not read); C cannot be packed."""
    buf = ctypes.create_string_buffer(256)
    d = gu.make_desc(mg.DTYPE_F64, 8, 8, 8, 1.0, 0.0, (ctypes.addressof(buf), 0, 0), (1, 1, 8), (1, 1, 8))
    d.a.mem = mg.MEM_PACKED
    assert lib.momms_gemm_validate(ctypes.byref(d)) == mg.ERR_INVALID_ARG
    assert b"packed" in lib.momms_last_error()
    d2 = gu.make_desc(mg.DTYPE_F64, 8, 8, 8, 1.0, 0.0, (1, 1, 8), (1, 1, 8), (ctypes.addressof(buf), 0, 0))
    d2.c.mem = mg.MEM_PACKED
    assert lib.momms_gemm_validate(ctypes.byref(d2)) == mg.ERR_INVALID_ARG
    assert lib.momms_packed_destroy(ctypes.c_void_p(ctypes.addressof(buf))) == mg.ERR_INVALID_ARG
    assert lib.momms_packed_bytes(ctypes.c_void_p(ctypes.addressof(buf))) == 0


def test_fault_injection_counters_without_a_gpu(lib):
    """The injection hook is plain host state: set, read back, cleared."""
    assert lib.momms_fault_inject(mg.FAULT_ALLOC, 3) == mg.OK
    assert lib.momms_fault_pending(mg.FAULT_ALLOC) == 3
    assert lib.momms_fault_pending(mg.FAULT_CUDA) == 0
    assert lib.momms_fault_inject(mg.FAULT_ALLOC, 0) == mg.OK
    assert lib.momms_fault_pending(mg.FAULT_ALLOC) == 0
    assert lib.momms_fault_inject(9, 1) == mg.ERR_INVALID_ARG
    assert lib.momms_fault_inject(mg.FAULT_CUDA, -1) == mg.ERR_INVALID_ARG
    assert lib.momms_fault_pending(9) == -1


def test_no_cpu_fallback(lib, tmp_path):
    """Without a GPU every compute mode returns MOMMS_ERR_NO_DEVICE and leaves
    C untouched (nothing is computed on the host), and a missing library is
    an ImportError, not a silent fallback."""
    import numpy as np
    if _torch_cuda():
        pytest.skip("a GPU is present")
    A = np.asfortranarray(np.ones((4, 3)))
    B = np.asfortranarray(np.ones((3, 5)))
    C = np.asfortranarray(np.full((4, 5), 7.0))

    def trip(x):
        return (x.ctypes.data, x.strides[0] // x.itemsize, x.strides[1] // x.itemsize)

    for dt, prec in ((mg.DTYPE_F64, mg.PREC_PLAIN), (mg.DTYPE_F64, mg.PREC_OZAKI)):
        d = gu.make_desc(dt, 4, 5, 3, 1.0, 1.0, trip(A), trip(B), trip(C), precision=prec, mem=mg.MEM_HOST)
        assert lib.momms_gemm(ctypes.byref(d), None) == mg.ERR_NO_DEVICE
        assert np.all(C == 7.0)
    A32, B32, C32 = (np.asfortranarray(x.astype(np.float32)) for x in (A, B, C))
    for prec in (mg.PREC_PLAIN, mg.PREC_SPLIT_TF32):
        d = gu.make_desc(mg.DTYPE_F32, 4, 5, 3, 1.0, 1.0, trip(A32), trip(B32), trip(C32), precision=prec,
                         mem=mg.MEM_HOST)
        assert lib.momms_gemm(ctypes.byref(d), None) == mg.ERR_NO_DEVICE
        assert np.all(C32 == 7.0)
    with pytest.raises(ImportError, match="no CPU fallback"):
        mg.load_library(path=str(tmp_path / "libmomms_gpu.so"))


def _torch_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def test_integration_notes_bind_every_function():
    """INTEGRATION.md shows the binding of every function include/*.h declares."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [n for n in declared_functions() if not re.search(r"\b%s\b" % n, text)]
    assert not missing, missing
