"""momms_gb300: the GB300 (sm_103a) blocked matrix multiply C := beta*C + alpha*A*B.

The product is the shared library ``libmomms_gpu.so`` built from ``csrc/``;
its C ABI is ``include/momms_gpu.h`` and the reference's view-based
``GemmNode`` interface over it is ``include/momms/gemm_node.hpp`` (C++). This
package loads the library for Python callers through ctypes, with the C
structs mirrored below. There is no CPU fallback: if the library is missing,
loading it raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmomms_gpu.so")

# momms_status
OK = 0
ERR_INVALID_ARG = 1
ERR_UNSUPPORTED = 2
ERR_CUDA = 3
ERR_NO_DEVICE = 4
ERR_OUT_OF_MEMORY = 5
ERR_DEVICE_TIMEOUT = 6
ERR_ADMISSION = 7
ERR_BUSY = 8
ERR_SHUTDOWN = 9
ERR_TARGET_UNREACHABLE = 10

KERNEL_DGEMM_DMMA = 0
KERNEL_SGEMM_FFMA = 1
KERNEL_SLICE_OZAKI = 2
KERNEL_SLICE_TF32 = 3
KERNEL_PREP = 4
KERNEL_COMBINE = 5
KERNEL_BOUND = 6
KERNEL_CLASSES = 7

FAULT_ALLOC = 0
FAULT_CUDA = 1

DTYPE_F64 = 0
DTYPE_F32 = 1
PREC_PLAIN = 0
PREC_OZAKI = 1
PREC_SPLIT_TF32 = 2
MEM_AUTO = 0
MEM_HOST = 1
MEM_DEVICE = 2
MEM_PACKED = 3
ROLE_A = 0
ROLE_B = 1


class Operand(ctypes.Structure):
    _fields_ = [("ptr", ctypes.c_void_p), ("rs", ctypes.c_int64), ("cs", ctypes.c_int64),
                ("mem", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class GemmDesc(ctypes.Structure):
    _fields_ = [("dtype", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("k", ctypes.c_int64),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double),
                ("a", Operand), ("b", Operand), ("c", Operand),
                ("target_rel_err", ctypes.c_double), ("slices", ctypes.c_int32),
                ("flags", ctypes.c_int32)]


class CallInfo(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("slices", ctypes.c_int32), ("pairs", ctypes.c_int32),
                ("groups", ctypes.c_int32), ("splits", ctypes.c_int32), ("slice_variant", ctypes.c_int32),
                ("bound_rel_err", ctypes.c_double)]


class TuneResult(ctypes.Structure):
    _fields_ = [("splits", ctypes.c_int32), ("candidates", ctypes.c_int32), ("best_ms", ctypes.c_float),
                ("tile", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_batch", ctypes.c_int32), ("max_inflight", ctypes.c_int32),
                ("queue_capacity", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("submit_s", ctypes.c_double), ("start_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("status", ctypes.c_int32), ("batch_size", ctypes.c_int32), ("batch_id", ctypes.c_uint64),
                ("device_start_ms", ctypes.c_double), ("device_end_ms", ctypes.c_double)]


class ServerReport(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("batches", ctypes.c_uint64), ("mean_batch", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("flops_completed", ctypes.c_double), ("busy_s", ctypes.c_double),
                ("tflops", ctypes.c_double), ("admitted_bytes", ctypes.c_uint64)]


class MommsError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"momms status {status}: {message}")
        self.status = status


_lib = None


def load_library(path=None):
    """Load (once) and return the ctypes handle of libmomms_gpu.so."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: build it with `python -m momms_gb300.build` "
                          "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(p)
    vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.momms_gemm.argtypes = [ctypes.POINTER(GemmDesc), vp]
    lib.momms_gemm.restype = i32
    lib.momms_gemm_validate.argtypes = [ctypes.POINTER(GemmDesc)]
    lib.momms_gemm_validate.restype = i32
    for name, ct in (("momms_dgemm", ctypes.c_double), ("momms_sgemm", ctypes.c_float)):
        f = getattr(lib, name)
        P = ctypes.POINTER(ct)
        f.argtypes = [i64, i64, i64, P, vp, i64, i64, vp, i64, i64, P, vp, i64, i64, vp]
        f.restype = i32
    Pd = ctypes.POINTER(ctypes.c_double)
    lib.momms_dgemm_noalloc.argtypes = [i64, i64, i64, Pd, vp, i64, i64, vp, i64, i64, Pd, vp, i64, i64, vp]
    lib.momms_dgemm_noalloc.restype = i32
    lib.momms_device_status.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    lib.momms_device_status.restype = i32
    lib.momms_noalloc_status.argtypes = [ctypes.POINTER(ctypes.c_uint32)]
    lib.momms_noalloc_status.restype = i32
    lib.momms_selftest_wait_expiry.argtypes = [ctypes.c_uint32, i32, vp]
    lib.momms_selftest_wait_expiry.restype = i32
    lib.momms_fault_inject.argtypes = [i32, i32]
    lib.momms_fault_inject.restype = i32
    lib.momms_fault_pending.argtypes = [i32]
    lib.momms_fault_pending.restype = i32
    lib.momms_status_string.argtypes = [i32]
    lib.momms_status_string.restype = ctypes.c_char_p
    lib.momms_last_error.argtypes = []
    lib.momms_last_error.restype = ctypes.c_char_p
    lib.momms_abi_version.argtypes = []
    lib.momms_abi_version.restype = i32
    lib.momms_launch_count.argtypes = []
    lib.momms_launch_count.restype = ctypes.c_ulonglong
    lib.momms_measure_peak.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    lib.momms_measure_peak.restype = i32
    PD = ctypes.POINTER(GemmDesc)
    lib.momms_plan_create.argtypes = [PD, i32, ctypes.POINTER(ctypes.c_void_p)]
    lib.momms_plan_create.restype = i32
    lib.momms_plan_launch.argtypes = [vp, vp]
    lib.momms_plan_launch.restype = i32
    lib.momms_plan_capture.argtypes = [vp, vp]
    lib.momms_plan_capture.restype = i32
    lib.momms_plan_destroy.argtypes = [vp]
    lib.momms_plan_destroy.restype = i32
    lib.momms_gemm_grouped.argtypes = [PD, i32, vp]
    lib.momms_gemm_grouped.restype = i32
    lib.momms_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
    lib.momms_server_create.restype = i32
    lib.momms_server_submit.argtypes = [vp, PD, ctypes.POINTER(ctypes.c_uint64)]
    lib.momms_server_submit.restype = i32
    lib.momms_server_poll.argtypes = [vp, ctypes.c_uint64, ctypes.POINTER(RequestInfo)]
    lib.momms_server_poll.restype = i32
    lib.momms_server_wait.argtypes = [vp, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(RequestInfo)]
    lib.momms_server_wait.restype = i32
    lib.momms_server_drain.argtypes = [vp, ctypes.c_double]
    lib.momms_server_drain.restype = i32
    lib.momms_server_stats.argtypes = [vp, ctypes.POINTER(ServerReport), i32]
    lib.momms_server_stats.restype = i32
    lib.momms_server_destroy.argtypes = [vp]
    lib.momms_server_destroy.restype = i32
    lib.momms_autotune.argtypes = [PD, ctypes.POINTER(TuneResult), vp]
    lib.momms_autotune.restype = i32
    lib.momms_autotune_batch.argtypes = [PD, i32, vp, ctypes.POINTER(ctypes.c_int32)]
    lib.momms_autotune_batch.restype = i32
    lib.momms_tune_export.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    lib.momms_tune_export.restype = i32
    lib.momms_tune_import.argtypes = [ctypes.c_char_p]
    lib.momms_tune_import.restype = i32
    lib.momms_tune_clear.argtypes = []
    lib.momms_tune_clear.restype = i32
    lib.momms_last_info.argtypes = [ctypes.POINTER(CallInfo)]
    lib.momms_last_info.restype = i32
    lib.momms_timing_enable.argtypes = [i32]
    lib.momms_timing_enable.restype = i32
    lib.momms_timing_read.argtypes = [i32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_ulonglong), i32]
    lib.momms_timing_read.restype = i32
    lib.momms_set_staging_budget.argtypes = [ctypes.c_uint64]
    lib.momms_set_staging_budget.restype = i32
    lib.momms_staging_budget.argtypes = []
    lib.momms_staging_budget.restype = ctypes.c_uint64
    i64p = ctypes.POINTER(ctypes.c_int64)
    lib.momms_stream_plan.argtypes = [PD, ctypes.c_uint64, i64p, i64p, i64p]
    lib.momms_stream_plan.restype = i32
    lib.momms_pack.argtypes = [i32, i32, i32, i64, i64, ctypes.POINTER(Operand), i32, vp, ctypes.POINTER(vp)]
    lib.momms_pack.restype = i32
    lib.momms_packed_destroy.argtypes = [vp]
    lib.momms_packed_destroy.restype = i32
    lib.momms_packed_bytes.argtypes = [vp]
    lib.momms_packed_bytes.restype = ctypes.c_uint64
    if path is None:
        _lib = lib
    return lib


def check(status, lib=None):
    """Raise MommsError for a non-zero status."""
    if status != OK:
        lib = lib or load_library()
        raise MommsError(status, lib.momms_last_error().decode() or lib.momms_status_string(status).decode())
    return status
