// Plain f64 GEMM on the FP64 tensor-core MMA (DMMA, mma.sync m8n8k4.f64).
//
// Replaces the reference's PackA/PackB copiers (src/composables/pack.rs:51-133)
// with TMA loads of 128B-swizzled tiles into a 4-stage shared-memory ring, its
// PartM/PartN/ParallelN loops (src/composables/part.rs:7-79,
// src/composables/parallel_range.rs:130-154) with a persistent CTA-tile
// scheduler, its PartK slabs (part.rs:81-120) with an in-register k loop plus
// optional split-k, and the d6x8 microkernel
// (ukernels/bli_gemm_haswell_asm_d6x8.c:666-1200) with warp-level DMMA.
//
// The epilogue keeps the microkernel's order: acc is scaled by alpha and then
// c = fma(beta, c, acc); beta == 0 stores without reading C (d6x8.c:889-1192).
// Unlike the reference, C is rounded once per element, not once per KC=192
// slab; both stay inside |dC| <= 2k u (|A||B|).
//
// One warp is the TMA producer, eight warps compute a 128 x 128 tile
// (warp tile 64 x 32 = 32 independent 8x8 accumulators). At GB300's FP64 rate
// (about 1 TFLOP/s per GPU) this shape keeps the DMMA pipe full; shared-memory
// traffic is about 1% of its bandwidth, so residual bank conflicts cost nothing
// measurable.
#include <stdio.h>

#include "dmma_core.cuh"
#include "internal.h"

namespace momms {
namespace dmma {

struct Params {
  int64_t m, n, k;
  double alpha, beta;
  double* c;
  int64_t rsc, csc;
  TileSched sched;
  double* partials;    // splits > 1: [tiles][splits][BM*BN]
  unsigned* counters;  // splits > 1: [tiles], zero on entry and on exit
  unsigned* status;
};

template <bool A_XC, bool B_XC>
__global__ void __launch_bounds__(THREADS, 1)
    dgemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const Params p) {
  extern __shared__ uint8_t smem_raw[];
  const Smem sm = setup_smem(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t units = p.sched.units();
  const int64_t kblocks = ceil_div_dev(p.k, BK);
  const int64_t kb_split = p.sched.k_per_split / BK;
  int stage = 0;
  uint32_t phase = 0;

  if (warp == CONSUMER_WARPS) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
        int tm, tn, sp;
        p.sched.decode(u, tm, tn, sp);
        const int64_t kb0 = sp * kb_split;
        const int64_t kb1 = min(kblocks, kb0 + kb_split);
        if (!produce_unit(&tmA, &tmB, A_XC, B_XC, tm, tn, kb0, kb1, sm.sA, sm.sB, sm.full, sm.empty, stage, phase,
                          p.status))
          return;
      }
    }
    return;
  }

  // ---------------- DMMA consumers ----------------
  const int wm = warp >> 2;  // 0..1 -> rows wm*64
  const int wn = warp & 3;   // 0..3 -> cols wn*32
  const Epi e{p.m, p.n, p.alpha, p.beta, p.c, p.rsc, p.csc};
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    int tm, tn, sp;
    p.sched.decode(u, tm, tn, sp);
    const int64_t kb0 = sp * kb_split;
    const int64_t kb1 = min(kblocks, kb0 + kb_split);
    const int64_t row_base = (int64_t)tm * BM + wm * 64, col_base = (int64_t)tn * BN + wn * 32;
    const uint32_t live = live_mask(row_base, col_base, p.m, p.n);
    double acc[8][4][2];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
    if (!consume_unit(A_XC, B_XC, kb0, kb1, live, sm.sA, sm.sB, sm.full, sm.empty, stage, phase, wm, wn, lane, acc,
                      p.status))
      return;
    const int64_t tile = u / p.sched.splits;
    finish_unit(e, acc, row_base + (lane >> 2), col_base + 2 * (lane & 3), p.sched.splits, sp,
                p.partials ? p.partials + (size_t)tile * p.sched.splits * BM * BN : nullptr,
                p.counters ? p.counters + tile : nullptr, threadIdx.x, sm.s_last);
  }
}

}  // namespace dmma

// ---------------------------------------------------------------------------
// Host launcher
// ---------------------------------------------------------------------------

namespace {

// Orientation of an operand for TMA: x-contiguous (the non-k index has unit
// stride), k-contiguous, or needs a repack.
enum Orient { ORIENT_XC, ORIENT_KC, ORIENT_REPACK };

// rows x cols operand where `x_is_rows` says whether the non-k index is the
// row index (A: rows = m) or the column index (B: cols = n).
Orient pick_orient(const DevMat& v, int64_t rows, int64_t cols, bool x_is_rows, size_t elem) {
  if ((reinterpret_cast<uintptr_t>(v.ptr) & 15) != 0) return ORIENT_REPACK;
  const int64_t vec = 16 / (int64_t)elem;
  const int64_t x_stride = x_is_rows ? v.rs : v.cs;
  const int64_t k_stride = x_is_rows ? v.cs : v.rs;
  const int64_t x_ext = x_is_rows ? rows : cols;
  const int64_t k_ext = x_is_rows ? cols : rows;
  if (x_stride == 1 && (k_ext == 1 || (k_stride > 0 && k_stride % vec == 0 && k_stride >= x_ext)))
    return ORIENT_XC;
  if (k_stride == 1 && (x_ext == 1 || (x_stride > 0 && x_stride % vec == 0 && x_stride >= k_ext)))
    return ORIENT_KC;
  return ORIENT_REPACK;
}

}  // namespace

int dmma_orient(const DevMat& v, int64_t rows, int64_t cols, bool x_is_rows) {
  return (int)pick_orient(v, rows, cols, x_is_rows, 8);
}

int set_attrs_dmma() {
  using namespace dmma;
  const void* kerns[4] = {(const void*)dgemm_kernel<true, true>, (const void*)dgemm_kernel<true, false>,
                          (const void*)dgemm_kernel<false, true>, (const void*)dgemm_kernel<false, false>};
  for (const void* kf : kerns) {
    cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(dgemm)");
  }
  return MOMMS_OK;
}

namespace {
// The launcher proper; scratch[0..2] (repacked A, B, split-k workspace) are
// returned to the pool by the caller, on every path.
int dgemm_dmma_impl(const DevGemm& g0, cudaStream_t s, void* (&scratch)[3]) {
  using namespace dmma;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  DevGemm g = g0;
  cudaError_t ce;
  if ((ce = wait_operands(g, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");

  // A: rows m, cols k, x = m. B: rows k, cols n, x = n.
  Orient oa = pick_orient(g.a, g.m, g.k, true, 8);
  Orient ob = pick_orient(g.b, g.k, g.n, false, 8);
  if (oa == ORIENT_REPACK) {
    int64_t ld = round_up(g.m, 2);
    if ((ce = scratch_alloc(&scratch[0], (size_t)ld * g.k * 8, s)) != cudaSuccess) return cuda_fail(ce, "scratch A");
    int rc = repack_colmajor(g.a, g.m, g.k, 8, scratch[0], ld, s);
    if (rc) return rc;
    g.a = DevMat{scratch[0], 1, ld};
    oa = ORIENT_XC;
  }
  if (ob == ORIENT_REPACK) {
    int64_t ld = round_up(g.k, 2);
    if ((ce = scratch_alloc(&scratch[1], (size_t)ld * g.n * 8, s)) != cudaSuccess) return cuda_fail(ce, "scratch B");
    int rc = repack_colmajor(g.b, g.k, g.n, 8, scratch[1], ld, s);
    if (rc) return rc;
    g.b = DevMat{scratch[1], 1, ld};
    ob = ORIENT_KC;
  }

  CUtensorMap tmA, tmB;
  {
    uint64_t dims[2], strides[1];
    uint32_t box[2];
    if (oa == ORIENT_XC) {
      dims[0] = g.m; dims[1] = g.k;
      strides[0] = (uint64_t)(g.k == 1 ? round_up(g.m * 8, 16) : g.a.cs * 8);
      box[0] = 16; box[1] = BK;
    } else {
      dims[0] = g.k; dims[1] = g.m;
      strides[0] = (uint64_t)(g.m == 1 ? round_up(g.k * 8, 16) : g.a.rs * 8);
      box[0] = BK; box[1] = BM;
    }
    int rc = encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, g.a.ptr, dims, strides, box,
                          CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    if (ob == ORIENT_XC) {
      dims[0] = g.n; dims[1] = g.k;
      strides[0] = (uint64_t)(g.k == 1 ? round_up(g.n * 8, 16) : g.b.rs * 8);
      box[0] = 16; box[1] = BK;
    } else {
      dims[0] = g.k; dims[1] = g.n;
      strides[0] = (uint64_t)(g.n == 1 ? round_up(g.k * 8, 16) : g.b.cs * 8);
      box[0] = BK; box[1] = BN;
    }
    rc = encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, g.b.ptr, dims, strides, box,
                      CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
  }

  Params p;
  p.m = g.m; p.n = g.n; p.k = g.k;
  p.alpha = g.alpha; p.beta = g.beta;
  p.c = static_cast<double*>(g.c.ptr);
  p.rsc = g.c.rs; p.csc = g.c.cs;
  p.status = ds->status;
  const int tiles_m = (int)ceil_div(g.m, BM), tiles_n = (int)ceil_div(g.n, BN);
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  const int64_t kblocks = ceil_div(g.k, BK);
  // Split k only when the output tiles cannot fill the GPU (each split keeps
  // at least two k-blocks; splits_f64).
  int splits = splits_f64(g.m, g.n, g.k, ds->sm_count);
  int64_t kb_split = ceil_div(kblocks, splits);
  splits = (int)ceil_div(kblocks, kb_split);
  p.sched = TileSched{tiles_m, tiles_n, splits, 8, kb_split * BK};
  call_info().splits = splits;
  p.partials = nullptr;
  p.counters = nullptr;
  void*& ws = scratch[2];
  if (splits > 1) {
    size_t part_bytes = (size_t)tiles * splits * BM * BN * 8;
    size_t cnt_bytes = (size_t)tiles * 4;
    if ((ce = scratch_alloc(&ws, part_bytes + cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "split-k workspace");
    p.partials = static_cast<double*>(ws);
    p.counters = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + part_bytes);
    if ((ce = cudaMemsetAsync(p.counters, 0, cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "memset counters");
  }

  const int64_t units = p.sched.units();
  const int grid = (int)std::min<int64_t>(units, ds->sm_count);
  auto launch = [&](auto kern) -> cudaError_t {
    {
      KernelTimer kt(MOMMS_KERNEL_DGEMM_DMMA, s);
      kern<<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
    }
    note_launch();
    return launch_status();
  };
  if (oa == ORIENT_XC && ob == ORIENT_XC) ce = launch(dgemm_kernel<true, true>);
  else if (oa == ORIENT_XC) ce = launch(dgemm_kernel<true, false>);
  else if (ob == ORIENT_XC) ce = launch(dgemm_kernel<false, true>);
  else ce = launch(dgemm_kernel<false, false>);
  if (ce != cudaSuccess) return cuda_fail(ce, "dgemm_dmma launch");
  return MOMMS_OK;
}
}  // namespace

int launch_dgemm_dmma(const DevGemm& g, cudaStream_t s) {
  void* scratch[3] = {nullptr, nullptr, nullptr};
  const int rc = dgemm_dmma_impl(g, s, scratch);
  // back to the pool in stream order, after the kernel if it was launched
  for (void* q : scratch)
    if (q) cudaFreeAsync(q, s);
  return rc;
}

}  // namespace momms

// ---------------------------------------------------------------------------
// momms_dgemm_noalloc: the f64 GEMM for callers that cannot allocate device
// memory. Same kernel and same tile / split-k plan as momms_dgemm on device
// operands; the split-k scratch comes from a fixed device-global array instead
// of the stream-ordered pool.
// ---------------------------------------------------------------------------
#include <mutex>

namespace momms {
namespace {

constexpr size_t kNoallocPartialTiles = 160;  // 128 x 128 f64 partial tiles
constexpr size_t kNoallocPartialBytes = kNoallocPartialTiles * dmma::BM * dmma::BN * sizeof(double);
constexpr size_t kNoallocCounterSlots = 1024;  // per-output-tile arrival counters
static_assert(kNoallocPartialBytes + kNoallocCounterSlots * sizeof(unsigned) == MOMMS_NOALLOC_SCRATCH_BYTES,
              "scratch layout must match MOMMS_NOALLOC_SCRATCH_BYTES");

// The scratch itself. Every GPU that loads this library holds these bytes
// until the process exits; every call of momms_dgemm_noalloc on a device uses
// the same bytes. In host code this name is only a stand-in for the device
// address: host code passes the address from cudaGetSymbolAddress instead.
static __device__ __align__(256) unsigned char g_noalloc_scratch[MOMMS_NOALLOC_SCRATCH_BYTES];
// The no-alloc calls' status word: a kernel whose bounded wait expires ORs a
// DEV_* bit in here (momms_noalloc_status reads and clears it). Like the
// scratch, one word per device for the life of the process.
static __device__ unsigned g_noalloc_status;

struct NoallocDevice {
  bool ready = false;
  void* scratch = nullptr;   // device address of g_noalloc_scratch on this device
  unsigned* status = nullptr;  // device address of g_noalloc_status on this device
  int sm_count = 0;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

// One-time set-up per device, run by the first call on that device with the
// device current: looks up the scratch array's device address and the SM
// count, and raises the kernels' shared-memory limit. Allocates nothing.
int noalloc_setup(NoallocDevice*& out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(MOMMS_ERR_NO_DEVICE, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoallocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
    void* st = nullptr;
    e = cudaGetSymbolAddress(&st, g_noalloc_status);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc status)");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    const void* kerns[4] = {(const void*)dmma::dgemm_kernel<true, true>, (const void*)dmma::dgemm_kernel<true, false>,
                            (const void*)dmma::dgemm_kernel<false, true>, (const void*)dmma::dgemm_kernel<false, false>};
    for (const void* kf : kerns) {
      e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, dmma::SMEM_BYTES);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    }
    d.scratch = p;
    d.status = static_cast<unsigned*>(st);
    d.sm_count = sms;
    d.ready = true;
  }
  out = &d;
  return MOMMS_OK;
}

}  // namespace

// The no-alloc status word of the current device (nullptr with the error
// recorded if the set-up fails); used by the wait-expiry self-test.
unsigned* noalloc_status_word() {
  NoallocDevice* nd = nullptr;
  return noalloc_setup(nd) ? nullptr : nd->status;
}
}  // namespace momms

extern "C" int momms_dgemm_noalloc(int64_t m, int64_t n, int64_t k, const double* alpha, const double* a,
                                   int64_t rs_a, int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b,
                                   const double* beta, double* c, int64_t rs_c, int64_t cs_c, void* stream) {
  using namespace momms;
  using namespace momms::dmma;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!alpha || !beta) return fail(MOMMS_ERR_INVALID_ARG, "alpha/beta pointer is null");
  if (m < 0 || n < 0 || k < 0) return fail(MOMMS_ERR_INVALID_ARG, "negative size");
  if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX) return fail(MOMMS_ERR_INVALID_ARG, "dimension above 2^31-1");
  if (m == 0 || n == 0 || k == 0) return MOMMS_OK;  // as momms_dgemm: k == 0 leaves C as it is
  if (!a || !b || !c) return fail(MOMMS_ERR_INVALID_ARG, "null operand pointer");
  if (rs_a < 0 || cs_a < 0 || rs_b < 0 || cs_b < 0 || rs_c < 0 || cs_c < 0)
    return fail(MOMMS_ERR_INVALID_ARG, "negative stride");
  if (m > 1 && n > 1 && rs_c == cs_c) return fail(MOMMS_ERR_INVALID_ARG, "C has equal strides");
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) {
    cudaGetLastError();
    return fail(MOMMS_ERR_NO_DEVICE, "no current CUDA device");
  }
  const void* ptrs[3] = {a, b, c};
  for (const void* p : ptrs) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
        !(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return fail(MOMMS_ERR_INVALID_ARG,
                  "momms_dgemm_noalloc takes device operands only (staging host memory would allocate)");
    }
    // the kernels' TMA reads go to this device's memory only
    if (at.type == cudaMemoryTypeDevice && at.device != cur)
      return fail(MOMMS_ERR_INVALID_ARG, "operand is memory of device %d, the current device is %d", at.device,
                  cur);
  }
  NoallocDevice* nd = nullptr;
  int rc = noalloc_setup(nd);
  if (rc) return rc;

  DevGemm g;
  g.dtype = MOMMS_DTYPE_F64;
  g.m = m; g.n = n; g.k = k;
  g.alpha = *alpha; g.beta = *beta;
  g.a = DevMat{const_cast<double*>(a), rs_a, cs_a};
  g.b = DevMat{const_cast<double*>(b), rs_b, cs_b};
  g.c = DevMat{c, rs_c, cs_c};
  const Orient oa = pick_orient(g.a, g.m, g.k, true, 8);
  const Orient ob = pick_orient(g.b, g.k, g.n, false, 8);
  if (oa == ORIENT_REPACK || ob == ORIENT_REPACK)
    return fail(MOMMS_ERR_INVALID_ARG,
                "momms_dgemm_noalloc needs A and B with unit stride along one index, the other stride a multiple of "
                "2 elements and 16-byte aligned bases (other layouts need a repack copy, which would allocate)");

  CUtensorMap tmA, tmB;
  {
    uint64_t dims[2], strides[1];
    uint32_t box[2];
    if (oa == ORIENT_XC) {
      dims[0] = g.m; dims[1] = g.k;
      strides[0] = (uint64_t)(g.k == 1 ? round_up(g.m * 8, 16) : g.a.cs * 8);
      box[0] = 16; box[1] = BK;
    } else {
      dims[0] = g.k; dims[1] = g.m;
      strides[0] = (uint64_t)(g.m == 1 ? round_up(g.k * 8, 16) : g.a.rs * 8);
      box[0] = BK; box[1] = BM;
    }
    rc = encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, g.a.ptr, dims, strides, box,
                      CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    if (ob == ORIENT_XC) {
      dims[0] = g.n; dims[1] = g.k;
      strides[0] = (uint64_t)(g.k == 1 ? round_up(g.n * 8, 16) : g.b.rs * 8);
      box[0] = 16; box[1] = BK;
    } else {
      dims[0] = g.k; dims[1] = g.n;
      strides[0] = (uint64_t)(g.n == 1 ? round_up(g.k * 8, 16) : g.b.cs * 8);
      box[0] = BK; box[1] = BN;
    }
    rc = encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, g.b.ptr, dims, strides, box,
                      CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
  }

  // The same tile / split-k plan as momms_dgemm, so both give the same result.
  Params p;
  p.m = g.m; p.n = g.n; p.k = g.k;
  p.alpha = g.alpha; p.beta = g.beta;
  p.c = c;
  p.rsc = rs_c; p.csc = cs_c;
  p.status = nd->status;  // the no-alloc status word, not the library's allocated one
  const int tiles_m = (int)ceil_div(g.m, BM), tiles_n = (int)ceil_div(g.n, BN);
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  const int64_t kblocks = ceil_div(g.k, BK);
  int splits = splits_f64(g.m, g.n, g.k, nd->sm_count);
  const int64_t kb_split = ceil_div(kblocks, splits);
  splits = (int)ceil_div(kblocks, kb_split);
  p.sched = TileSched{tiles_m, tiles_n, splits, 8, kb_split * BK};
  p.partials = nullptr;
  p.counters = nullptr;
  if (splits > 1) {
    if ((size_t)(tiles * splits) > kNoallocPartialTiles || (size_t)tiles > kNoallocCounterSlots)
      return fail(MOMMS_ERR_INVALID_ARG,
                  "this problem needs %lld split-k partial tiles of 128x128 doubles; the no-alloc scratch holds %zu "
                  "(%d bytes)",
                  (long long)(tiles * splits), kNoallocPartialTiles, (int)MOMMS_NOALLOC_SCRATCH_BYTES);
    p.partials = static_cast<double*>(nd->scratch);
    p.counters = reinterpret_cast<unsigned*>(static_cast<unsigned char*>(nd->scratch) + kNoallocPartialBytes);
    // counters must start at zero; the array keeps whatever the last call left
    cudaError_t e = cudaMemsetAsync(p.counters, 0, (size_t)tiles * sizeof(unsigned), s);
    if (e != cudaSuccess) return cuda_fail(e, "clear split-k counters");
  }
  const int grid = (int)std::min<int64_t>(p.sched.units(), nd->sm_count);
  if (oa == ORIENT_XC && ob == ORIENT_XC) dgemm_kernel<true, true><<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
  else if (oa == ORIENT_XC) dgemm_kernel<true, false><<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
  else if (ob == ORIENT_XC) dgemm_kernel<false, true><<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
  else dgemm_kernel<false, false><<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
  note_launch();
  cudaError_t e = launch_status();
  if (e != cudaSuccess) return cuda_fail(e, "dgemm_noalloc launch");
  return MOMMS_OK;
}

extern "C" int momms_noalloc_status(uint32_t* bits) {
  using namespace momms;
  NoallocDevice* nd = nullptr;
  int rc = noalloc_setup(nd);
  if (rc) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceSynchronize");
  unsigned w = 0;
  const unsigned zero = 0;
  e = cudaMemcpyFromSymbol(&w, g_noalloc_status, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_noalloc_status, &zero, sizeof(unsigned));
  if (e != cudaSuccess) return cuda_fail(e, "no-alloc status word");
  if (bits) *bits = w;
  if (w) return fail(MOMMS_ERR_DEVICE_TIMEOUT, "no-alloc status bits 0x%x", w);
  return MOMMS_OK;
}
