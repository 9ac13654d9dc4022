// The C ABI of include/momms_gpu.h: argument checks, memory-space detection,
// host<->device staging, dispatch to the kernels, error reporting.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace momms {

namespace {
thread_local char g_last_error[512] = "";
thread_local momms_call_info g_info;
thread_local momms_call_info g_last_info;
std::mutex g_dev_mu;
DeviceState g_devices[64];
}  // namespace

momms_call_info& call_info() { return g_info; }

namespace {
std::atomic<int> g_fault_pending[2];
}  // namespace

bool fault_take(int kind) {
  if (kind < 0 || kind > 1) return false;
  int n = g_fault_pending[kind].load();
  while (n > 0)
    if (g_fault_pending[kind].compare_exchange_weak(n, n - 1)) return true;
  return false;
}

cudaError_t device_malloc(void** ptr, size_t bytes) {
  if (fault_take(MOMMS_FAULT_ALLOC)) return cudaErrorMemoryAllocation;
  return cudaMalloc(ptr, bytes);
}

namespace {
thread_local cudaError_t g_refused_launch = cudaSuccess;
}  // namespace

void refuse_launch(cudaError_t e) { g_refused_launch = e; }

cudaError_t launch_status() {
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && g_refused_launch != cudaSuccess) e = g_refused_launch;
  g_refused_launch = cudaSuccess;
  if (e == cudaSuccess && fault_take(MOMMS_FAULT_CUDA)) e = cudaErrorLaunchFailure;
  return e;
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear a sticky-free error so the next call starts clean
  if (e == cudaErrorMemoryAllocation) return fail(MOMMS_ERR_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return fail(MOMMS_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
  return fail(MOMMS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

DeviceState* device_state() {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    cuda_fail(e == cudaSuccess ? cudaErrorInvalidDevice : e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(g_dev_mu);
  DeviceState& d = g_devices[dev];
  if (d.device < 0) {
    int sms = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
      cuda_fail(e, "cudaDeviceGetAttribute");
      return nullptr;
    }
    unsigned* st = nullptr;
    if ((e = cudaMalloc(&st, sizeof(unsigned))) != cudaSuccess) {
      cuda_fail(e, "status word");
      return nullptr;
    }
    if ((e = cudaMemset(st, 0, sizeof(unsigned))) != cudaSuccess) {
      cuda_fail(e, "status word");
      return nullptr;
    }
    int rc = set_attrs_dmma();
    if (!rc) rc = set_attrs_grouped();
    if (!rc) rc = set_attrs_tf32();
    if (!rc) rc = set_attrs_ozaki();
    if (rc) return nullptr;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) {
      cuda_fail(e, "scratch pool");
      return nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    cudaStream_t cs = nullptr, cs2 = nullptr, aux = nullptr, aux2 = nullptr;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&aux2, cudaStreamNonBlocking)) != cudaSuccess) {
      cuda_fail(e, "library stream");
      return nullptr;
    }
    d.copy_stream = cs;
    d.copy_stream2 = cs2;
    d.aux = aux;
    d.aux2 = aux2;
    d.pool = pool;
    d.sm_count = sms;
    d.status = st;
    d.device = dev;
  }
  return &d;
}

cudaError_t scratch_alloc_raw(void** ptr, size_t bytes, cudaStream_t s) {
  if (fault_take(MOMMS_FAULT_ALLOC)) return cudaErrorMemoryAllocation;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    cs = cudaStreamCaptureStatusNone;
  }
  DeviceState* d = (cs == cudaStreamCaptureStatusNone) ? device_state() : nullptr;
  if (d && d->pool) return cudaMallocFromPoolAsync(ptr, bytes, d->pool, s);
  return cudaMallocAsync(ptr, bytes, s);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, uint32_t rank, const void* gaddr, const uint64_t* dims,
                 const uint64_t* strides_bytes, const uint32_t* box, CUtensorMapSwizzle swizzle) {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  if (!fn) return fail(MOMMS_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(map, dtype, rank, const_cast<void*>(gaddr), dims, strides_bytes, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return fail(MOMMS_ERR_INVALID_ARG, "cuTensorMapEncodeTiled failed (%d) rank=%u dims=%llu,%llu box=%u,%u", (int)r,
                rank, (unsigned long long)dims[0], (unsigned long long)(rank > 1 ? dims[1] : 0), box[0],
                rank > 1 ? box[1] : 0);
  return MOMMS_OK;
}

// ---------------------------------------------------------------------------
// Repack a strided operand into column-major scratch.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void repack_kernel(const T* __restrict__ src, int64_t rs, int64_t cs, int64_t rows, int64_t cols,
                              T* __restrict__ dst, int64_t ld) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % rows, j = e / rows;
    dst[i + j * ld] = src[i * rs + j * cs];
  }
}

int repack_colmajor(const DevMat& src, int64_t rows, int64_t cols, size_t elem, void* dst, int64_t ld,
                    cudaStream_t s) {
  const int64_t total = rows * cols;
  if (total == 0) return MOMMS_OK;
  const int threads = 256;
  const int blocks = (int)std::min<int64_t>(ceil_div(total, threads), 4096);
  KernelTimer kt(MOMMS_KERNEL_PREP, s);
  if (elem == 8)
    repack_kernel<double><<<blocks, threads, 0, s>>>(static_cast<const double*>(src.ptr), src.rs, src.cs, rows, cols,
                                                      static_cast<double*>(dst), ld);
  else
    repack_kernel<float><<<blocks, threads, 0, s>>>(static_cast<const float*>(src.ptr), src.rs, src.cs, rows, cols,
                                                     static_cast<float*>(dst), ld);
  note_launch();
  cudaError_t e = launch_status();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "repack");
}

// ---------------------------------------------------------------------------
// Validation and staging
// ---------------------------------------------------------------------------
namespace {

size_t elem_size(int dtype) { return dtype == MOMMS_DTYPE_F64 ? 8 : 4; }

int validate(const momms_gemm_desc* d) {
  if (!d) return fail(MOMMS_ERR_INVALID_ARG, "desc is null");
  if (d->dtype != MOMMS_DTYPE_F64 && d->dtype != MOMMS_DTYPE_F32)
    return fail(MOMMS_ERR_INVALID_ARG, "unknown dtype %d", d->dtype);
  if (d->precision < MOMMS_PREC_PLAIN || d->precision > MOMMS_PREC_SPLIT_TF32)
    return fail(MOMMS_ERR_INVALID_ARG, "unknown precision %d", d->precision);
  if (d->precision == MOMMS_PREC_OZAKI && d->dtype != MOMMS_DTYPE_F64)
    return fail(MOMMS_ERR_UNSUPPORTED, "Ozaki emulation is an f64 mode");
  if (d->precision == MOMMS_PREC_SPLIT_TF32 && d->dtype != MOMMS_DTYPE_F32)
    return fail(MOMMS_ERR_UNSUPPORTED, "split-TF32 is an f32 mode");
  if (d->precision == MOMMS_PREC_OZAKI && (d->slices < 0 || d->slices > kOzakiMaxSlices))
    return fail(MOMMS_ERR_INVALID_ARG, "Ozaki slice count %d outside 0..16", d->slices);
  if (d->precision == MOMMS_PREC_OZAKI && !(d->target_rel_err >= 0.0 && d->target_rel_err < 1.0))
    return fail(MOMMS_ERR_INVALID_ARG, "target_rel_err must be in [0, 1)");
  if (d->m < 0 || d->n < 0 || d->k < 0) return fail(MOMMS_ERR_INVALID_ARG, "negative size m=%lld n=%lld k=%lld",
                                                    (long long)d->m, (long long)d->n, (long long)d->k);
  if (d->m > INT32_MAX || d->n > INT32_MAX || d->k > INT32_MAX)
    return fail(MOMMS_ERR_INVALID_ARG, "dimension above 2^31-1");
  if (d->flags != 0) return fail(MOMMS_ERR_INVALID_ARG, "flags must be 0");
  const momms_operand* ops[3] = {&d->a, &d->b, &d->c};
  const int64_t rows[3] = {d->m, d->k, d->m}, cols[3] = {d->k, d->n, d->n};
  const char* names = "ABC";
  for (int i = 0; i < 3; ++i) {
    if (rows[i] == 0 || cols[i] == 0) continue;
    if (i < 2 && (d->m == 0 || d->n == 0)) continue;
    if (!ops[i]->ptr) return fail(MOMMS_ERR_INVALID_ARG, "%c.ptr is null", names[i]);
    if (ops[i]->mem == MOMMS_MEM_PACKED) {
      if (i == 2) return fail(MOMMS_ERR_INVALID_ARG, "C cannot be a packed operand");
      const int rc = check_packed(*d, i, packed_of(*ops[i]));
      if (rc) return rc;
      continue;
    }
    if (ops[i]->rs < 0 || ops[i]->cs < 0) return fail(MOMMS_ERR_INVALID_ARG, "%c has a negative stride", names[i]);
    if ((rows[i] > 1 && ops[i]->rs == 0) || (cols[i] > 1 && ops[i]->cs == 0))
      return fail(MOMMS_ERR_INVALID_ARG, "%c has a zero stride", names[i]);
    if (ops[i]->mem < MOMMS_MEM_AUTO || ops[i]->mem > MOMMS_MEM_PACKED)
      return fail(MOMMS_ERR_INVALID_ARG, "%c.mem is not a momms_memspace", names[i]);
  }
  // C must not overlap itself: the strides must separate rows and columns.
  if (d->m > 1 && d->n > 1 && d->c.rs == d->c.cs) return fail(MOMMS_ERR_INVALID_ARG, "C has equal strides");
  return MOMMS_OK;
}

// Per-call staging state: the hooks the launchers see, the copy streams
// (host->device on `copy`, device->host on `back`) and the call's events
// (ev 0-2: A, B, C copied in; 3: buffers allocated; 4, 5: copy streams done).
struct StagedCall {
  Staging hooks;
  cudaStream_t copy = nullptr, back = nullptr;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> col_ev;  // column copies (deferred operands) and write-back ranges
  const momms_operand* ops[3] = {nullptr, nullptr, nullptr};
  const Staged* st = nullptr;
  size_t es = 0;
  ~StagedCall() {
    for (cudaEvent_t e : col_ev) cudaEventDestroy(e);
  }
  cudaError_t new_event(cudaEvent_t* e) {
    cudaError_t r = cudaEventCreateWithFlags(e, cudaEventDisableTiming);
    if (r == cudaSuccess) col_ev.push_back(*e);
    return r;
  }
};

int writeback_cols(Staging* h, int64_t j0, int64_t j1, cudaStream_t s) {
  StagedCall* sc = static_cast<StagedCall*>(h->ctx);
  cudaEvent_t ev = nullptr;
  cudaError_t e = sc->new_event(&ev);
  if (e == cudaSuccess) e = cudaEventRecord(ev, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(sc->back, ev, 0);
  if (e != cudaSuccess) return cuda_fail(e, "C copy-back");
  return stage_out_cols(*sc->ops[2], sc->es, sc->st[2], j0, j1, sc->back);
}

int copy_cols_in(Staging* h, int which, int64_t j0, int64_t j1, cudaEvent_t* done) {
  StagedCall* sc = static_cast<StagedCall*>(h->ctx);
  int rc = stage_in_cols(*sc->ops[which], sc->es, sc->st[which], j0, j1, sc->copy);
  if (rc || !done) return rc;
  cudaError_t e = sc->new_event(done);
  if (e == cudaSuccess) e = cudaEventRecord(*done, sc->copy);
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "staging events");
}

int dispatch(const DevGemm& g, const momms_gemm_desc* d, cudaStream_t s) {
  if (g.dtype == MOMMS_DTYPE_F64) {
    if (d->precision == MOMMS_PREC_OZAKI) {
      int used = 0;
      return launch_dgemm_ozaki(g, d->target_rel_err, d->slices, &used, s);
    }
    return launch_dgemm_dmma(g, s);
  }
  if (d->precision == MOMMS_PREC_SPLIT_TF32) return launch_sgemm_tf32x3(g, s);
  return launch_sgemm_ffma(g, s);
}

}  // namespace

int run_device_gemm(const DevGemm& g, const momms_gemm_desc& d, cudaStream_t s) { return dispatch(g, &d, s); }

int gemm_impl(const momms_gemm_desc* d, cudaStream_t s) {
  g_last_error[0] = 0;
  int rc = validate(d);
  if (rc) return rc;
  // The reference's PartK loop runs no slab when k == 0 and leaves C as it
  // is (src/composables/part.rs:98-106); so does this node.
  if (d->m == 0 || d->n == 0 || d->k == 0) return MOMMS_OK;
  if (!device_state()) return MOMMS_ERR_NO_DEVICE;
  memset(&g_info, 0, sizeof(g_info));
  g_info.precision = d->precision;
  g_info.bound_rel_err = -1.0;
  const size_t es = elem_size(d->dtype);
  const momms_operand* ops[3] = {&d->a, &d->b, &d->c};
  const int64_t rows[3] = {d->m, d->k, d->m}, cols[3] = {d->k, d->n, d->n};
  bool host[3];
  for (int i = 0; i < 3; ++i)
    host[i] = ops[i]->mem == MOMMS_MEM_HOST || (ops[i]->mem == MOMMS_MEM_AUTO && !is_device_ptr(ops[i]->ptr));
  const bool any_packed = packed_of(d->a) || packed_of(d->b);
  const bool any_host0 = host[0] || host[1] || host[2];
  if (any_host0) {
    // Larger than the staging budget: stream the operands through in blocks
    // (the reference's out-of-core PartM / PartN, src/exper/out_of_core.rs:77-87).
    const uint64_t budget = staging_budget();
    if (incore_bytes(*d, host) > budget) {
      if (any_packed) return fail(MOMMS_ERR_UNSUPPORTED, "streamed (out-of-core) calls take no packed operands");
      BlockPlan plan;
      rc = plan_blocks(*d, host, budget, &plan);
      if (!rc) rc = gemm_streamed(*d, host, plan, s);
      if (!rc || rc == MOMMS_ERR_TARGET_UNREACHABLE) g_last_info = g_info;
      return rc;
    }
  }
  DevGemm g;
  g.dtype = d->dtype;
  g.m = d->m;
  g.n = d->n;
  g.k = d->k;
  g.alpha = d->alpha;
  g.beta = d->beta;
  Staged st[3];
  DevMat* dm[3] = {&g.a, &g.b, &g.c};
  const bool any_host = host[0] || host[1] || host[2];
  bool need[3];
  const DevGemm gv = devgemm_of(*d);  // device views; packed operands resolved
  g.pk[0] = gv.pk[0];
  g.pk[1] = gv.pk[1];
  const DevMat views[3] = {gv.a, gv.b, gv.c};
  for (int i = 0; i < 3; ++i) {
    need[i] = host[i] && (i < 2 || d->beta != 0.0);  // C is read only when beta != 0
    if (!host[i]) *dm[i] = views[i];
  }
  for (int i = 0; i < 3 && !rc; ++i)
    if (host[i]) {
      rc = stage_alloc(*ops[i], rows[i], cols[i], es, st[i], s);
      if (!rc) *dm[i] = st[i].dev;
    }

  // Staging overlap: the host->device copies run on the device's copy stream
  // while the kernels that do not need them yet run on `s`; C comes back per
  // column range. Not inside stream capture (the call synchronises anyway).
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (any_host && cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  DeviceState* ds = device_state();
  const bool overlap = any_host && cap == cudaStreamCaptureStatusNone && ds && ds->copy_stream;
  StagedCall sc;
  sc.copy = overlap ? ds->copy_stream : s;
  sc.back = overlap ? ds->copy_stream2 : s;
  for (int i = 0; i < 3; ++i) sc.ops[i] = ops[i];
  sc.st = st;
  sc.es = es;
  if (!rc && overlap) {
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&sc.ev[i], cudaEventDisableTiming);
    // the copy streams start after the staging buffers exist (allocated on s)
    if (e == cudaSuccess) e = cudaEventRecord(sc.ev[3], s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(sc.copy, sc.ev[3], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(sc.back, sc.ev[3], 0);
    if (e != cudaSuccess) rc = cuda_fail(e, "staging events");
    sc.hooks.ctx = &sc;
    sc.hooks.copy_cols = copy_cols_in;
    for (int i = 0; i < 3 && !rc; ++i)
      if (need[i]) {
        // The emulated path reads B and C by column ranges and enqueues
        // their copies itself, in the order it needs them.
        if (i > 0 && d->precision == MOMMS_PREC_OZAKI && plain_pitch(*ops[i], st[i])) {
          sc.hooks.deferred[i] = true;
          continue;
        }
        rc = stage_copy_in(*ops[i], es, st[i], sc.copy);
        if (!rc && (e = cudaEventRecord(sc.ev[i], sc.copy)) != cudaSuccess) rc = cuda_fail(e, "staging events");
        if (!rc) sc.hooks.ready[i] = sc.ev[i];
      }
    if (host[2] && plain_pitch(*ops[2], st[2])) sc.hooks.writeback = writeback_cols;
    g.staging = &sc.hooks;
  } else {
    for (int i = 0; i < 3 && !rc; ++i)
      if (need[i]) rc = stage_copy_in(*ops[i], es, st[i], s);
  }

  // an unreachable accuracy target still leaves a result in C: finish the
  // call (C's copy-back included) and report it at the end
  int verdict = MOMMS_OK;
  if (!rc) rc = dispatch(g, d, s);
  if (rc == MOMMS_ERR_TARGET_UNREACHABLE) {
    verdict = rc;
    rc = MOMMS_OK;
  }
  if (!rc && host[2]) {
    if (sc.hooks.writeback) rc = columns_done(g, sc.hooks.written, g.n, s);  // what the path left
    else rc = stage_out(*ops[2], es, st[2], s);
  }
  if (overlap && sc.ev[5]) {
    // s (and so the frees below) waits for everything on the copy streams
    cudaError_t e = cudaEventRecord(sc.ev[4], sc.copy);
    if (e == cudaSuccess) e = cudaEventRecord(sc.ev[5], sc.back);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, sc.ev[4], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, sc.ev[5], 0);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "staging events");
  }
  for (int i = 0; i < 3; ++i)
    if (st[i].owned) cudaFreeAsync(st[i].owned, s);
  if (any_host) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (!rc && e != cudaSuccess) rc = cuda_fail(e, "stream synchronize");
  }
  for (int i = 0; i < 6; ++i)
    if (sc.ev[i]) cudaEventDestroy(sc.ev[i]);
  if (!rc) {
    g_last_info = g_info;
    rc = verdict;
  }
  return rc;
}

}  // namespace momms

// ---------------------------------------------------------------------------
// extern "C" surface
// ---------------------------------------------------------------------------
extern "C" {

int momms_gemm(const momms_gemm_desc* desc, void* stream) {
  return momms::gemm_impl(desc, static_cast<cudaStream_t>(stream));
}

int momms_gemm_validate(const momms_gemm_desc* desc) {
  int rc = momms::validate(desc);
  return rc;
}

static momms_gemm_desc make_desc(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* a,
                                 int64_t rs_a, int64_t cs_a, const void* b, int64_t rs_b, int64_t cs_b, double beta,
                                 void* c, int64_t rs_c, int64_t cs_c) {
  momms_gemm_desc d;
  memset(&d, 0, sizeof(d));
  d.dtype = dtype;
  d.precision = MOMMS_PREC_PLAIN;
  d.m = m;
  d.n = n;
  d.k = k;
  d.alpha = alpha;
  d.beta = beta;
  d.a = momms_operand{const_cast<void*>(a), rs_a, cs_a, MOMMS_MEM_AUTO, 0};
  d.b = momms_operand{const_cast<void*>(b), rs_b, cs_b, MOMMS_MEM_AUTO, 0};
  d.c = momms_operand{c, rs_c, cs_c, MOMMS_MEM_AUTO, 0};
  return d;
}

int momms_dgemm(int64_t m, int64_t n, int64_t k, const double* alpha, const double* a, int64_t rs_a, int64_t cs_a,
                const double* b, int64_t rs_b, int64_t cs_b, const double* beta, double* c, int64_t rs_c,
                int64_t cs_c, void* stream) {
  if (!alpha || !beta) return momms::fail(MOMMS_ERR_INVALID_ARG, "alpha/beta pointer is null");
  momms_gemm_desc d = make_desc(MOMMS_DTYPE_F64, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c);
  return momms::gemm_impl(&d, static_cast<cudaStream_t>(stream));
}

int momms_sgemm(int64_t m, int64_t n, int64_t k, const float* alpha, const float* a, int64_t rs_a, int64_t cs_a,
                const float* b, int64_t rs_b, int64_t cs_b, const float* beta, float* c, int64_t rs_c, int64_t cs_c,
                void* stream) {
  if (!alpha || !beta) return momms::fail(MOMMS_ERR_INVALID_ARG, "alpha/beta pointer is null");
  momms_gemm_desc d = make_desc(MOMMS_DTYPE_F32, m, n, k, *alpha, a, rs_a, cs_a, b, rs_b, cs_b, *beta, c, rs_c, cs_c);
  return momms::gemm_impl(&d, static_cast<cudaStream_t>(stream));
}

int momms_device_status(uint32_t* bits) {
  momms::DeviceState* ds = momms::device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return momms::cuda_fail(e, "cudaDeviceSynchronize");
  unsigned w = 0;
  e = cudaMemcpy(&w, ds->status, sizeof(unsigned), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemset(ds->status, 0, sizeof(unsigned));
  if (e != cudaSuccess) return momms::cuda_fail(e, "status word");
  if (bits) *bits = w;
  if (w) return momms::fail(MOMMS_ERR_DEVICE_TIMEOUT, "device status bits 0x%x", w);
  return MOMMS_OK;
}

int momms_fault_inject(int kind, int count) {
  if (kind != MOMMS_FAULT_ALLOC && kind != MOMMS_FAULT_CUDA)
    return momms::fail(MOMMS_ERR_INVALID_ARG, "unknown fault kind %d", kind);
  if (count < 0) return momms::fail(MOMMS_ERR_INVALID_ARG, "negative fault count");
  momms::g_fault_pending[kind].store(count);
  return MOMMS_OK;
}

int momms_fault_pending(int kind) {
  if (kind != MOMMS_FAULT_ALLOC && kind != MOMMS_FAULT_CUDA) return -1;
  return momms::g_fault_pending[kind].load();
}

const char* momms_status_string(int status) {
  switch (status) {
    case MOMMS_OK: return "ok";
    case MOMMS_ERR_INVALID_ARG: return "invalid argument";
    case MOMMS_ERR_UNSUPPORTED: return "unsupported dtype/precision combination";
    case MOMMS_ERR_CUDA: return "CUDA runtime error";
    case MOMMS_ERR_NO_DEVICE: return "no usable CUDA device";
    case MOMMS_ERR_OUT_OF_MEMORY: return "device out of memory";
    case MOMMS_ERR_DEVICE_TIMEOUT: return "a kernel's bounded wait expired";
    case MOMMS_ERR_ADMISSION: return "request exceeds the admission budget";
    case MOMMS_ERR_BUSY: return "busy";
    case MOMMS_ERR_SHUTDOWN: return "server stopped";
    case MOMMS_ERR_TARGET_UNREACHABLE: return "requested accuracy cannot be guaranteed with 15 slices";
    default: return "unknown status";
  }
}

const char* momms_last_error(void) { return momms::g_last_error; }

int momms_abi_version(void) { return MOMMS_ABI_VERSION; }

int momms_last_info(momms_call_info* out) {
  if (!out) return momms::fail(MOMMS_ERR_INVALID_ARG, "out is null");
  *out = momms::g_last_info;
  return MOMMS_OK;
}

}  // extern "C"
