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

#include "common.cuh"
#include "internal.h"

namespace momms {
namespace dmma {

constexpr int BM = 128, BN = 128, BK = 16, STAGES = 4;
constexpr int CONSUMER_WARPS = 8;  // 2 (m) x 4 (n)
constexpr int THREADS = (CONSUMER_WARPS + 1) * 32;
constexpr int CONSUMERS = CONSUMER_WARPS * 32;
constexpr int A_STAGE = BM * BK * 8;  // bytes
constexpr int B_STAGE = BN * BK * 8;
constexpr int SUB = BK * 128;  // one 16-wide sub-tile of an x-contiguous operand
constexpr int SMEM_BYTES = 1024 + STAGES * (A_STAGE + B_STAGE) + 2 * STAGES * 8 + 16;

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

// Byte offset of element (r, kk) in a k-contiguous tile: rows of 16 doubles
// (128 bytes), 128B swizzle (16-byte chunk index XOR row mod 8).
__device__ __forceinline__ uint32_t off_kc(int r, int kk) {
  return r * 128 + ((((kk >> 1) ^ (r & 7))) << 4) + ((kk & 1) << 3);
}
// Byte offset of element (x, kk) in an x-contiguous tile stored as BM/16
// sub-tiles of [BK rows of k][16 doubles of x], each 128B-swizzled.
__device__ __forceinline__ uint32_t off_xc(int x, int kk) {
  return (x >> 4) * SUB + kk * 128 + (((((x & 15) >> 1) ^ (kk & 7))) << 4) + ((x & 1) << 3);
}

__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}

__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, %0;" ::"n"(CONSUMERS) : "memory"); }

__device__ __forceinline__ void store_c(const Params& p, int64_t row, int64_t col, double v) {
  if (row < p.m && col < p.n) {
    double* cp = p.c + row * p.rsc + col * p.csc;
    double s = v * p.alpha;
    *cp = (p.beta == 0.0) ? s : fma(p.beta, *cp, s);
  }
}

template <bool A_XC, bool B_XC>
__global__ void __launch_bounds__(THREADS, 1)
    dgemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const Params p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + STAGES * B_STAGE);
  uint64_t* empty = full + STAGES;
  int* s_last = reinterpret_cast<int*>(empty + STAGES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], CONSUMER_WARPS);
    }
    fence_barrier_init();
  }
  __syncthreads();

  const int64_t units = p.sched.units();
  const int64_t kblocks = ceil_div_dev(p.k, BK);
  const int64_t kb_split = p.sched.k_per_split / BK;

  if (warp == CONSUMER_WARPS) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      int stage = 0;
      uint32_t phase = 0;
      for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
        int tm, tn, sp;
        p.sched.decode(u, tm, tn, sp);
        const int64_t kb0 = sp * kb_split;
        const int64_t kb1 = min(kblocks, kb0 + kb_split);
        for (int64_t kb = kb0; kb < kb1; ++kb) {
          if (!mbar_wait_bounded(&empty[stage], phase ^ 1)) {
            report_status(p.status, DEV_TIMEOUT_EMPTY);
            return;
          }
          mbar_arrive_expect_tx(&full[stage], A_STAGE + B_STAGE);
          uint8_t* a_dst = sA + stage * A_STAGE;
          uint8_t* b_dst = sB + stage * B_STAGE;
          const int32_t kc = (int32_t)(kb * BK);
          if (A_XC) {
#pragma unroll
            for (int j = 0; j < BM / 16; ++j) tma_load_2d(a_dst + j * SUB, &tmA, &full[stage], tm * BM + 16 * j, kc);
          } else {
            tma_load_2d(a_dst, &tmA, &full[stage], kc, tm * BM);
          }
          if (B_XC) {
#pragma unroll
            for (int j = 0; j < BN / 16; ++j) tma_load_2d(b_dst + j * SUB, &tmB, &full[stage], tn * BN + 16 * j, kc);
          } else {
            tma_load_2d(b_dst, &tmB, &full[stage], kc, tn * BN);
          }
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
    }
    return;
  }

  // ---------------- DMMA consumers ----------------
  const int wm = warp >> 2;  // 0..1 -> rows wm*64
  const int wn = warp & 3;   // 0..3 -> cols wn*32
  const int ctid = threadIdx.x;
  int stage = 0;
  uint32_t phase = 0;
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    int tm, tn, sp;
    p.sched.decode(u, tm, tn, sp);
    const int64_t kb0 = sp * kb_split;
    const int64_t kb1 = min(kblocks, kb0 + kb_split);

    double acc[8][4][2];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    for (int64_t kb = kb0; kb < kb1; ++kb) {
      if (!mbar_wait_bounded(&full[stage], phase)) {
        report_status(p.status, DEV_TIMEOUT_FULL);
        return;
      }
      const uint8_t* a = sA + stage * A_STAGE;
      const uint8_t* b = sB + stage * B_STAGE;
#pragma unroll
      for (int ks = 0; ks < BK / 4; ++ks) {
        const int kk = ks * 4 + (lane & 3);
        double af[8], bf[4];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int r = wm * 64 + i * 8 + (lane >> 2);
          af[i] = *reinterpret_cast<const double*>(a + (A_XC ? off_xc(r, kk) : off_kc(r, kk)));
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int cidx = wn * 32 + j * 8 + (lane >> 2);
          bf[j] = *reinterpret_cast<const double*>(b + (B_XC ? off_xc(cidx, kk) : off_kc(cidx, kk)));
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[stage]);
      if (++stage == STAGES) {
        stage = 0;
        phase ^= 1;
      }
    }

    const int64_t row0 = (int64_t)tm * BM + wm * 64 + (lane >> 2);
    const int64_t col0 = (int64_t)tn * BN + wn * 32 + 2 * (lane & 3);
    if (p.sched.splits == 1) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int e = 0; e < 2; ++e) store_c(p, row0 + i * 8, col0 + j * 8 + e, acc[i][j][e]);
    } else {
      // Split-k: publish this split's partial tile; the last split to
      // arrive sums all partials in split order 0..S-1 (a fixed order, so the
      // result does not depend on which CTA finishes last) and writes C.
      const int64_t tile = u / p.sched.splits;
      const size_t tile_elems = (size_t)BM * BN;
      double* part = p.partials + ((size_t)tile * p.sched.splits + sp) * tile_elems;
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int e = 0; e < 2; ++e) part[((i * 4 + j) * 2 + e) * CONSUMERS + ctid] = acc[i][j][e];
      __threadfence();
      consumer_sync();
      if (ctid == 0) {
        unsigned prev = atomicAdd(&p.counters[tile], 1u);
        *s_last = (prev == (unsigned)(p.sched.splits - 1)) ? 1 : 0;
      }
      consumer_sync();
      if (*s_last) {
        __threadfence();
        const double* base = p.partials + (size_t)tile * p.sched.splits * tile_elems;
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
              const int r = ((i * 4 + j) * 2 + e) * CONSUMERS + ctid;
              double s = __ldcg(base + r);
              for (int q = 1; q < p.sched.splits; ++q) s += __ldcg(base + (size_t)q * tile_elems + r);
              store_c(p, row0 + i * 8, col0 + j * 8 + e, s);
            }
        if (ctid == 0) p.counters[tile] = 0u;
      }
      consumer_sync();
    }
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

int launch_dgemm_dmma(const DevGemm& g0, cudaStream_t s) {
  using namespace dmma;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  DevGemm g = g0;
  void* scratch[2] = {nullptr, nullptr};
  cudaError_t ce;

  // A: rows m, cols k, x = m. B: rows k, cols n, x = n.
  Orient oa = pick_orient(g.a, g.m, g.k, true, 8);
  Orient ob = pick_orient(g.b, g.k, g.n, false, 8);
  if (oa == ORIENT_REPACK) {
    int64_t ld = round_up(g.m, 2);
    if ((ce = cudaMallocAsync(&scratch[0], (size_t)ld * g.k * 8, s)) != cudaSuccess) return cuda_fail(ce, "scratch A");
    int rc = repack_colmajor(g.a, g.m, g.k, 8, scratch[0], ld, s);
    if (rc) return rc;
    g.a = DevMat{scratch[0], 1, ld};
    oa = ORIENT_XC;
  }
  if (ob == ORIENT_REPACK) {
    int64_t ld = round_up(g.k, 2);
    if ((ce = cudaMallocAsync(&scratch[1], (size_t)ld * g.n * 8, s)) != cudaSuccess) return cuda_fail(ce, "scratch B");
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
  // Split k only when the output tiles cannot fill the GPU; each split keeps
  // at least 8 k-blocks.
  int splits = 1;
  if (tiles < ds->sm_count) {
    splits = (int)std::min<int64_t>(ds->sm_count / tiles, kblocks / 8);
    splits = std::max(1, std::min(splits, 32));
  }
  int64_t kb_split = ceil_div(kblocks, splits);
  splits = (int)ceil_div(kblocks, kb_split);
  p.sched = TileSched{tiles_m, tiles_n, splits, 8, kb_split * BK};
  call_info().splits = splits;
  p.partials = nullptr;
  p.counters = nullptr;
  void* ws = nullptr;
  if (splits > 1) {
    size_t part_bytes = (size_t)tiles * splits * BM * BN * 8;
    size_t cnt_bytes = (size_t)tiles * 4;
    if ((ce = cudaMallocAsync(&ws, part_bytes + cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "split-k workspace");
    p.partials = static_cast<double*>(ws);
    p.counters = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + part_bytes);
    if ((ce = cudaMemsetAsync(p.counters, 0, cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "memset counters");
  }

  const int64_t units = p.sched.units();
  const int grid = (int)std::min<int64_t>(units, ds->sm_count);
  auto launch = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (e != cudaSuccess) return e;
    {
      KernelTimer kt(MOMMS_KERNEL_DGEMM_DMMA, s);
      kern<<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB, p);
    }
    note_launch();
    return cudaGetLastError();
  };
  if (oa == ORIENT_XC && ob == ORIENT_XC) ce = launch(dgemm_kernel<true, true>);
  else if (oa == ORIENT_XC) ce = launch(dgemm_kernel<true, false>);
  else if (ob == ORIENT_XC) ce = launch(dgemm_kernel<false, true>);
  else ce = launch(dgemm_kernel<false, false>);
  if (ce != cudaSuccess) return cuda_fail(ce, "dgemm_dmma launch");
  if (ws) cudaFreeAsync(ws, s);
  for (void* q : scratch)
    if (q) cudaFreeAsync(q, s);
  return MOMMS_OK;
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

struct NoallocDevice {
  bool ready = false;
  void* scratch = nullptr;  // device address of g_noalloc_scratch on this device
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
    d.sm_count = sms;
    d.ready = true;
  }
  out = &d;
  return MOMMS_OK;
}

}  // namespace
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
  const void* ptrs[3] = {a, b, c};
  for (const void* p : ptrs) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
        !(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)) {
      cudaGetLastError();
      return fail(MOMMS_ERR_INVALID_ARG,
                  "momms_dgemm_noalloc takes device operands only (staging host memory would allocate)");
    }
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
  p.status = nullptr;  // no status word here: that one is allocated on first use
  const int tiles_m = (int)ceil_div(g.m, BM), tiles_n = (int)ceil_div(g.n, BN);
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  const int64_t kblocks = ceil_div(g.k, BK);
  int splits = 1;
  if (tiles < nd->sm_count) {
    splits = (int)std::min<int64_t>(nd->sm_count / tiles, kblocks / 8);
    splits = std::max(1, std::min(splits, 32));
  }
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
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "dgemm_noalloc launch");
  return MOMMS_OK;
}
