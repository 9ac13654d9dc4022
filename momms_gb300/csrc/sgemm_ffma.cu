// Plain f32 GEMM on the FP32 pipes: register-blocked FFMA.
//
// The GPU form of the reference's f32 path (the bli_sgemm_haswell_asm_6x16
// register block, ukernels/bli_gemm_haswell_asm_d6x8.c:77-640, under the same
// Goto loops): a persistent 128 x 128 CTA tile, 256 threads each owning an
// 8 x 8 register block, k streamed in blocks of 8 through double-buffered
// shared memory. Global loads are 128-bit and coalesced along whichever index
// of the operand is contiguous; k-contiguous operands are transposed on their
// way into shared memory so that every inner-loop read is a conflict-free
// 128-bit load. Each output element is a sequential fma chain over k (the
// microkernel's order, d6x8.c:725-885), then acc*alpha, then
// fma(beta, c, acc).
#include "common.cuh"
#include "internal.h"

namespace momms {
namespace ffma {

constexpr int BM = 128, BN = 128, BK = 8, THREADS = 256;

struct Params {
  int64_t m, n, k;
  float alpha, beta;
  const float* a;
  int64_t rsa, csa;
  const float* b;
  int64_t rsb, csb;
  float* c;
  int64_t rsc, csc;
  TileSched sched;
  float* partials;
  unsigned* counters;
};

__device__ __forceinline__ void store_c(const Params& p, int64_t row, int64_t col, float v) {
  if (row < p.m && col < p.n) {
    float* cp = p.c + row * p.rsc + col * p.csc;
    float s = v * p.alpha;
    *cp = (p.beta == 0.0f) ? s : fmaf(p.beta, *cp, s);
  }
}

// Loads 4 elements of an operand: `x` (the non-k index) and `kk` give the
// first element; the 4 elements run along the contiguous index when CONTIG_X
// (x, x+1, x+2, x+3) or along k otherwise (kk .. kk+3).
template <bool VEC, bool ALONG_X>
__device__ __forceinline__ float4 load4(const float* base, int64_t sx, int64_t sk, int64_t x, int64_t kk, int64_t xe,
                                        int64_t ke) {
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  const bool full = ALONG_X ? (x + 3 < xe && kk < ke) : (x < xe && kk + 3 < ke);
  if (VEC && full) {
    v = __ldg(reinterpret_cast<const float4*>(base + x * sx + kk * sk));
  } else {
    float t[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t xi = ALONG_X ? x + i : x;
      const int64_t ki = ALONG_X ? kk : kk + i;
      t[i] = (xi < xe && ki < ke) ? __ldg(base + xi * sx + ki * sk) : 0.f;
    }
    v = make_float4(t[0], t[1], t[2], t[3]);
  }
  return v;
}

template <bool A_XC, bool B_XC, bool VEC>
__global__ void __launch_bounds__(THREADS, 2) sgemm_kernel(const Params p) {
  __shared__ __align__(16) float As[2][BK][BM];
  __shared__ __align__(16) float Bs[2][BK][BN];
  __shared__ int s_last;

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  // load assignment
  const int ax = A_XC ? (tid & 31) * 4 : (tid >> 1);
  const int ak = A_XC ? (tid >> 5) : (tid & 1) * 4;
  const int bx = B_XC ? (tid & 31) * 4 : (tid >> 1);
  const int bk = B_XC ? (tid >> 5) : (tid & 1) * 4;

  const int64_t units = p.sched.units();
  const int64_t kblocks = ceil_div_dev(p.k, BK);
  const int64_t kb_split = p.sched.k_per_split / BK;

  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    int tm, tn, sp;
    p.sched.decode(u, tm, tn, sp);
    const int64_t kb0 = sp * kb_split;
    const int64_t kb1 = min(kblocks, kb0 + kb_split);
    const int64_t m0 = (int64_t)tm * BM, n0 = (int64_t)tn * BN;
    // (x, k) element strides of A (x = m) and B (x = n)
    const float* abase = p.a + m0 * p.rsa;
    const float* bbase = p.b + n0 * p.csb;
    const int64_t me = p.m - m0, ne = p.n - n0;

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    float4 ra, rb;
    auto gload = [&](int64_t kb) {
      const int64_t k0 = kb * BK;
      ra = load4<VEC, A_XC>(abase + k0 * p.csa, p.rsa, p.csa, ax, ak, me, p.k - k0);
      rb = load4<VEC, B_XC>(bbase + k0 * p.rsb, p.csb, p.rsb, bx, bk, ne, p.k - k0);
    };
    auto sstore = [&](int buf) {
      if (A_XC) {
        *reinterpret_cast<float4*>(&As[buf][ak][ax]) = ra;
      } else {
        As[buf][ak + 0][ax] = ra.x;
        As[buf][ak + 1][ax] = ra.y;
        As[buf][ak + 2][ax] = ra.z;
        As[buf][ak + 3][ax] = ra.w;
      }
      if (B_XC) {
        *reinterpret_cast<float4*>(&Bs[buf][bk][bx]) = rb;
      } else {
        Bs[buf][bk + 0][bx] = rb.x;
        Bs[buf][bk + 1][bx] = rb.y;
        Bs[buf][bk + 2][bx] = rb.z;
        Bs[buf][bk + 3][bx] = rb.w;
      }
    };

    if (kb0 < kb1) {
      gload(kb0);
      sstore(0);
      __syncthreads();
      for (int64_t kb = kb0; kb < kb1; ++kb) {
        const int buf = (int)((kb - kb0) & 1);
        const bool more = kb + 1 < kb1;
        if (more) gload(kb + 1);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
          const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
          const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
          const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
          const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
          const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
          const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
          for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (more) sstore(buf ^ 1);
        __syncthreads();
      }
    }

    auto row_of = [&](int i) -> int64_t { return m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4)); };
    auto col_of = [&](int j) -> int64_t { return n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4)); };
    if (p.sched.splits == 1) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) store_c(p, row_of(i), col_of(j), acc[i][j]);
    } else {
      const int64_t tile = u / p.sched.splits;
      const size_t tile_elems = (size_t)BM * BN;
      float* part = p.partials + ((size_t)tile * p.sched.splits + sp) * tile_elems;
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) part[(i * 8 + j) * THREADS + tid] = acc[i][j];
      __threadfence();
      __syncthreads();
      if (tid == 0) {
        unsigned prev = atomicAdd(&p.counters[tile], 1u);
        s_last = (prev == (unsigned)(p.sched.splits - 1)) ? 1 : 0;
      }
      __syncthreads();
      if (s_last) {
        __threadfence();
        const float* base = p.partials + (size_t)tile * p.sched.splits * tile_elems;
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int r = (i * 8 + j) * THREADS + tid;
            float s = __ldcg(base + r);
            for (int q = 1; q < p.sched.splits; ++q) s += __ldcg(base + (size_t)q * tile_elems + r);
            store_c(p, row_of(i), col_of(j), s);
          }
        if (tid == 0) p.counters[tile] = 0u;
      }
      __syncthreads();
    }
  }
}

}  // namespace ffma

int launch_sgemm_ffma(const DevGemm& g0, cudaStream_t s) {
  using namespace ffma;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  DevGemm g = g0;
  void* scratch[2] = {nullptr, nullptr};
  cudaError_t ce;
  // A must have unit stride along m or k; B along k or n. Anything else is
  // first copied into a column-major scratch matrix.
  auto unit = [](const DevMat& v, int64_t, int64_t) { return v.rs == 1 || v.cs == 1; };
  if (!unit(g.a, g.m, g.k)) {
    int64_t ld = round_up(g.m, 4);
    if ((ce = cudaMallocAsync(&scratch[0], (size_t)ld * g.k * 4, s)) != cudaSuccess) return cuda_fail(ce, "scratch A");
    int rc = repack_colmajor(g.a, g.m, g.k, 4, scratch[0], ld, s);
    if (rc) return rc;
    g.a = DevMat{scratch[0], 1, ld};
  }
  if (!unit(g.b, g.k, g.n)) {
    int64_t ld = round_up(g.k, 4);
    if ((ce = cudaMallocAsync(&scratch[1], (size_t)ld * g.n * 4, s)) != cudaSuccess) return cuda_fail(ce, "scratch B");
    int rc = repack_colmajor(g.b, g.k, g.n, 4, scratch[1], ld, s);
    if (rc) return rc;
    g.b = DevMat{scratch[1], 1, ld};
  }
  // Degenerate extents make both strides "unit"; normalise so that the
  // contiguous index is the one the kernel streams along.
  const bool a_xc = (g.a.rs == 1) && !(g.a.cs == 1 && g.m == 1);
  const bool b_xc = (g.b.cs == 1) && !(g.b.rs == 1 && g.n == 1);
  const int64_t a_ld = a_xc ? g.a.cs : g.a.rs;
  const int64_t b_ld = b_xc ? g.b.rs : g.b.cs;
  const bool vec = ((reinterpret_cast<uintptr_t>(g.a.ptr) | reinterpret_cast<uintptr_t>(g.b.ptr)) & 15) == 0 &&
                   (a_ld % 4 == 0) && (b_ld % 4 == 0);

  Params p;
  p.m = g.m; p.n = g.n; p.k = g.k;
  p.alpha = (float)g.alpha; p.beta = (float)g.beta;
  p.a = static_cast<const float*>(g.a.ptr); p.rsa = g.a.rs; p.csa = g.a.cs;
  p.b = static_cast<const float*>(g.b.ptr); p.rsb = g.b.rs; p.csb = g.b.cs;
  p.c = static_cast<float*>(g.c.ptr); p.rsc = g.c.rs; p.csc = g.c.cs;
  const int tiles_m = (int)ceil_div(g.m, BM), tiles_n = (int)ceil_div(g.n, BN);
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  const int64_t kblocks = ceil_div(g.k, BK);
  const int slots = ds->sm_count * 2;
  int splits = 1;
  if (tiles < slots) {
    splits = (int)std::min<int64_t>(slots / tiles, kblocks / 16);
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
    size_t part_bytes = (size_t)tiles * splits * BM * BN * 4;
    size_t cnt_bytes = (size_t)tiles * 4;
    if ((ce = cudaMallocAsync(&ws, part_bytes + cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "split-k workspace");
    p.partials = static_cast<float*>(ws);
    p.counters = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + part_bytes);
    if ((ce = cudaMemsetAsync(p.counters, 0, cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "memset counters");
  }
  const int grid = (int)std::min<int64_t>(p.sched.units(), slots);
  {
    KernelTimer kt(MOMMS_KERNEL_SGEMM_FFMA, s);
    if (a_xc && b_xc) {
      if (vec) sgemm_kernel<true, true, true><<<grid, THREADS, 0, s>>>(p);
      else sgemm_kernel<true, true, false><<<grid, THREADS, 0, s>>>(p);
    } else if (a_xc) {
      if (vec) sgemm_kernel<true, false, true><<<grid, THREADS, 0, s>>>(p);
      else sgemm_kernel<true, false, false><<<grid, THREADS, 0, s>>>(p);
    } else if (b_xc) {
      if (vec) sgemm_kernel<false, true, true><<<grid, THREADS, 0, s>>>(p);
      else sgemm_kernel<false, true, false><<<grid, THREADS, 0, s>>>(p);
    } else {
      if (vec) sgemm_kernel<false, false, true><<<grid, THREADS, 0, s>>>(p);
      else sgemm_kernel<false, false, false><<<grid, THREADS, 0, s>>>(p);
    }
  }
  note_launch();
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return cuda_fail(ce, "sgemm_ffma launch");
  if (ws) cudaFreeAsync(ws, s);
  for (void* q : scratch)
    if (q) cudaFreeAsync(q, s);
  return MOMMS_OK;
}

}  // namespace momms
