// Building blocks of the FP32 FFMA GEMM kernels (single-problem and grouped).
//
// A 128 x 128 CTA tile, 256 threads each owning an 8 x 8 register block, k
// streamed in blocks of 8 through double-buffered shared memory. Global loads
// are 128-bit and coalesced along whichever index of the operand is
// contiguous; k-contiguous operands are transposed on their way into shared
// memory so that every inner-loop read is a conflict-free 128-bit load. Each
// output element is a sequential fma chain over k (the order of the
// reference's register-blocked microkernel), then acc*alpha, then
// fma(beta, c, acc).
#pragma once
#include "common.cuh"

namespace momms {
namespace ffma {

constexpr int BM = 128, BN = 128, BK = 8, THREADS = 256;

// One operand pair and the problem extent.
struct Operands {
  const float* a;
  int64_t rsa, csa;
  const float* b;
  int64_t rsb, csb;
  int64_t m, n, k;
  bool a_xc, b_xc, vec;  // A m-contiguous, B n-contiguous, 16-byte vector loads allowed
};

struct Epi {
  int64_t m, n;
  float alpha, beta;
  float* c;
  int64_t rsc, csc;
};

__device__ __forceinline__ void store_c(const Epi& e, int64_t row, int64_t col, float v) {
  if (row < e.m && col < e.n) {
    float* cp = e.c + row * e.rsc + col * e.csc;
    float s = v * e.alpha;
    *cp = (e.beta == 0.0f) ? s : fmaf(e.beta, *cp, s);
  }
}

// Loads 4 elements of an operand: `x` (the non-k index) and `kk` give the
// first element; the 4 elements run along x when `along_x` (x .. x+3) or
// along k otherwise (kk .. kk+3).
__device__ __forceinline__ float4 load4(bool vec, bool along_x, const float* base, int64_t sx, int64_t sk, int64_t x,
                                        int64_t kk, int64_t xe, int64_t ke) {
  const bool full = along_x ? (x + 3 < xe && kk < ke) : (x < xe && kk + 3 < ke);
  if (vec && full) return __ldg(reinterpret_cast<const float4*>(base + x * sx + kk * sk));
  float t[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t xi = along_x ? x + i : x;
    const int64_t ki = along_x ? kk : kk + i;
    t[i] = (xi < xe && ki < ke) ? __ldg(base + xi * sx + ki * sk) : 0.f;
  }
  return make_float4(t[0], t[1], t[2], t[3]);
}

// Accumulates k-blocks [kb0, kb1) of output tile (tm, tn) into acc.
__device__ __forceinline__ void ffma_unit(const Operands& o, int tm, int tn, int64_t kb0, int64_t kb1,
                                          float (&acc)[8][8], float (*As)[BK][BM], float (*Bs)[BK][BN]) {
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int ax = o.a_xc ? (tid & 31) * 4 : (tid >> 1);
  const int ak = o.a_xc ? (tid >> 5) : (tid & 1) * 4;
  const int bx = o.b_xc ? (tid & 31) * 4 : (tid >> 1);
  const int bk = o.b_xc ? (tid >> 5) : (tid & 1) * 4;
  const int64_t m0 = (int64_t)tm * BM, n0 = (int64_t)tn * BN;
  const float* abase = o.a + m0 * o.rsa;
  const float* bbase = o.b + n0 * o.csb;
  const int64_t me = o.m - m0, ne = o.n - n0;
  float4 ra, rb;
  auto gload = [&](int64_t kb) {
    const int64_t k0 = kb * BK;
    ra = load4(o.vec, o.a_xc, abase + k0 * o.csa, o.rsa, o.csa, ax, ak, me, o.k - k0);
    rb = load4(o.vec, o.b_xc, bbase + k0 * o.rsb, o.csb, o.rsb, bx, bk, ne, o.k - k0);
  };
  auto sstore = [&](int buf) {
    if (o.a_xc) {
      *reinterpret_cast<float4*>(&As[buf][ak][ax]) = ra;
    } else {
      As[buf][ak + 0][ax] = ra.x;
      As[buf][ak + 1][ax] = ra.y;
      As[buf][ak + 2][ax] = ra.z;
      As[buf][ak + 3][ax] = ra.w;
    }
    if (o.b_xc) {
      *reinterpret_cast<float4*>(&Bs[buf][bk][bx]) = rb;
    } else {
      Bs[buf][bk + 0][bx] = rb.x;
      Bs[buf][bk + 1][bx] = rb.y;
      Bs[buf][bk + 2][bx] = rb.z;
      Bs[buf][bk + 3][bx] = rb.w;
    }
  };
  if (kb0 >= kb1) return;
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

__device__ __forceinline__ int64_t row_of(int tm, int i) {
  const int ty = threadIdx.x >> 4;
  return (int64_t)tm * BM + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
}
__device__ __forceinline__ int64_t col_of(int tn, int j) {
  const int tx = threadIdx.x & 15;
  return (int64_t)tn * BN + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
}

// Epilogue; split-k partials are summed by the last split in split order.
__device__ __forceinline__ void ffma_finish(const Epi& e, float (&acc)[8][8], int tm, int tn, int splits, int sp,
                                            float* tile_partials, unsigned* counter, int* s_last) {
  const int tid = threadIdx.x;
  if (splits == 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) store_c(e, row_of(tm, i), col_of(tn, j), acc[i][j]);
    return;
  }
  const size_t tile_elems = (size_t)BM * BN;
  float* part = tile_partials + (size_t)sp * tile_elems;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) part[(i * 8 + j) * THREADS + tid] = acc[i][j];
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    unsigned prev = atomicAdd(counter, 1u);
    *s_last = (prev == (unsigned)(splits - 1)) ? 1 : 0;
  }
  __syncthreads();
  if (*s_last) {
    __threadfence();
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int r = (i * 8 + j) * THREADS + tid;
        float s = __ldcg(tile_partials + r);
        for (int q = 1; q < splits; ++q) s += __ldcg(tile_partials + (size_t)q * tile_elems + r);
        store_c(e, row_of(tm, i), col_of(tn, j), s);
      }
    if (tid == 0) *counter = 0u;
  }
  __syncthreads();
}

}  // namespace ffma
}  // namespace momms
