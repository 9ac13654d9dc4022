// Building blocks of the FP32 FFMA GEMM kernels (single-problem and grouped).
//
// A 128 x 128 CTA tile, 256 threads each owning an 8 x 8 register block, k
// streamed in blocks of 16 through double-buffered shared memory (or a 64 x 64
// tile of 64 threads, below). The eight warps form a 2 (m) x 4 (n) grid of
// 64 x 32 warp tiles; a warp's lanes form
// an 8 (m) x 4 (n) grid of 4 x 4 blocks, each lane owning two such blocks in m
// (32 apart) and two in n (16 apart). So every fragment read of a k step is
// one 128-byte shared-memory wavefront (A: 8 distinct 16-byte rows per warp,
// B: 4). Global loads are 128-bit and coalesced along whichever index of the
// operand is contiguous; k-contiguous operands are transposed on their way
// into shared memory (their rows padded by 4 floats so that the transposing
// stores of the two k halves fall on different banks). Each output element is a
// sequential fma chain over k (the order of the reference's register-blocked
// microkernel), then acc*alpha, then fma(beta, c, acc).
//
// Measured on GB300 at m=n=k=8192 (column-major, 2 CTAs per SM, one kernel
// timed alone): 55.7 TFLOP/s, against 48.4 for the earlier 8-deep k-block,
// 16 x 16 thread grid, row-outer FMA order and 64-bit addressing; results are
// bit-identical (same fma chain). Shared memory is reached through pointers
// derived from the kernel's dynamic shared array (a reference to a static
// __shared__ struct measured 9 % slower).
#pragma once
#include "common.cuh"

namespace momms {
namespace ffma {

// Tiles: TM x TM with TM = 128 (2 x 4 warps, 256 threads) or 64 (1 x 2
// warps, 64 threads, for small problems: four times the CTAs per output
// area). Every thread owns an 8 x 8 register block and every output is the
// same fma chain over k in both, so the tile size never changes a result.
constexpr int BK = 16;
constexpr int BM = 128, BN = 128, THREADS = 256;  // the default (large) tile
template <int TM>
struct Tile {
  static constexpr int WM = TM / 64, WN = TM / 32;   // warp grid (64 x 32 warp tiles)
  static constexpr int THREADS = WM * WN * 32;
  static constexpr int SROW_MAX = TM + 4;
  static constexpr int SMEM_BYTES = 2 * 2 * BK * SROW_MAX * 4;
  static constexpr int CTAS_PER_SM = TM == 128 ? 2 : 8;
};
// Floats per shared-memory k row: TM, padded by 4 for a k-contiguous
// operand (its transposing stores of the two k halves then fall on different
// banks). An x-contiguous operand stays unpadded.
template <int TM, bool XC>
__host__ __device__ constexpr int srow() { return XC ? TM : TM + 4; }

// The 8 x 8 register block of this thread: rows row0 + {0..3, 32..35},
// columns col0 + {0..3, 16..19} of the CTA tile.
template <int TM>
__device__ __forceinline__ int row0() {
  return ((threadIdx.x >> 5) % Tile<TM>::WM) * 64 + (threadIdx.x & 7) * 4;
}
template <int TM>
__device__ __forceinline__ int col0() {
  return ((threadIdx.x >> 5) / Tile<TM>::WM) * 32 + ((threadIdx.x & 31) >> 3) * 4;
}
template <int TM>
__device__ __forceinline__ int row_in_tile(int i) { return row0<TM>() + (i < 4 ? i : 28 + i); }
template <int TM>
__device__ __forceinline__ int col_in_tile(int j) { return col0<TM>() + (j < 4 ? j : 12 + j); }

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

// Dynamic shared memory of the kernels: double-buffered k-block tiles of A
// and B, [operand][buffer][k][SROW_MAX] floats.
constexpr int SMEM_BYTES = Tile<128>::SMEM_BYTES;

// This thread's share of one operand's k-block: NV 4-element pieces, along x
// (the non-k index) for an x-contiguous operand, along k otherwise. The
// position is an element offset from the operand's base pointer, 32-bit when
// every offset of both operands fits (Off = uint32_t, the common case: it
// keeps the loop's address arithmetic narrow) and 64-bit otherwise.
template <int TM, bool XC, typename Off>
struct TileLoader {
  static constexpr int T = Tile<TM>::THREADS;
  // x-contiguous: TM/4 threads cover a k row; k-contiguous: T/TM threads share a row
  static constexpr int TPK = TM / 4, TPR = T / TM;
  static constexpr int JSTEP = XC ? T / TPK : 4 * TPR;  // k distance between a thread's pieces
  static constexpr int NV = BK / JSTEP;
  Off off;   // element (x, k) of the current k-block
  int x, k;  // tile coordinates of the first element
  __device__ __forceinline__ void init(Off ld, int64_t x0, int64_t k0) {
    const int t = threadIdx.x;
    x = XC ? (t % TPK) * 4 : (t / TPR);
    k = XC ? (t / TPK) : (t % TPR) * 4;
    off = XC ? (Off)(x0 + x) + (Off)(k0 + k) * ld : (Off)(x0 + x) * ld + (Off)(k0 + k);
  }
  // Loads the k-block; `checked` guards every element against the extents
  // (xl, kl: elements inside the tile along x and k, at most TM and 16) and
  // needs no alignment.
  __device__ __forceinline__ void load(const float* __restrict__ base, float4 (&r)[NV], Off ld, bool checked, int xl,
                                       int kl) const {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const float* q = base + (XC ? off + (Off)(JSTEP * j) * ld : off + (Off)(JSTEP * j));
      const int kj = k + JSTEP * j;
      if (!checked) {
        r[j] = __ldg(reinterpret_cast<const float4*>(q));
      } else {
        float t4[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const bool ok = XC ? (x + i < xl && kj < kl) : (x < xl && kj + i < kl);
          t4[i] = ok ? __ldg(q + i) : 0.f;
        }
        r[j] = make_float4(t4[0], t4[1], t4[2], t4[3]);
      }
    }
  }
  // s: one [BK][srow] buffer in shared memory
  __device__ __forceinline__ void store(float* s, const float4 (&r)[NV]) const {
    constexpr int S = srow<TM, XC>();
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      const int kj = k + JSTEP * j;
      if (XC) {
        *reinterpret_cast<float4*>(s + kj * S + x) = r[j];
      } else {
        s[(kj + 0) * S + x] = r[j].x;
        s[(kj + 1) * S + x] = r[j].y;
        s[(kj + 2) * S + x] = r[j].z;
        s[(kj + 3) * S + x] = r[j].w;
      }
    }
  }
};

// True when every element offset of both operands fits in 32 bits, so the
// kernels may use the narrow loader.
inline bool offsets_fit_32(const Operands& o) {
  const double lim = 4294967295.0;
  const double amax = (double)(o.m - 1) * (double)o.rsa + (double)(o.k - 1) * (double)o.csa + 16.0;
  const double bmax = (double)(o.k - 1) * (double)o.rsb + (double)(o.n - 1) * (double)o.csb + 16.0;
  return amax < lim && bmax < lim;
}

// Accumulates k-blocks [kb0, kb1) of output tile (tm, tn) into acc. `smem`
// is the kernel's dynamic shared memory (Tile<TM>::SMEM_BYTES), addressed
// here through pointers derived from it so that every access is a
// shared-memory one.
template <int TM, bool A_XC, bool B_XC, typename Off>
__device__ __forceinline__ void ffma_unit_t(const Operands& o, int tm, int tn, int64_t kb0, int64_t kb1,
                                            float (&acc)[8][8], float* smem) {
  if (kb0 >= kb1) return;
  constexpr int SA = srow<TM, A_XC>(), SB = srow<TM, B_XC>(), SRM = Tile<TM>::SROW_MAX;
  float(*As)[BK * SRM] = reinterpret_cast<float(*)[BK * SRM]>(smem);
  float(*Bs)[BK * SRM] = reinterpret_cast<float(*)[BK * SRM]>(smem + 2 * BK * SRM);
  const int64_t m0 = (int64_t)tm * TM, n0 = (int64_t)tn * TM;
  // extents clamped to the tile: exact for every in-tile comparison
  const int ml = (int)min(o.m - m0, (int64_t)TM), nl = (int)min(o.n - n0, (int64_t)TM);
  const bool interior = o.vec && ml == TM && nl == TM;
  const Off lda = (Off)(A_XC ? o.csa : o.rsa), ldb = (Off)(B_XC ? o.rsb : o.csb);
  const Off stepa = A_XC ? (Off)BK * lda : (Off)BK, stepb = B_XC ? (Off)BK * ldb : (Off)BK;
  const int nkb = (int)(kb1 - kb0);
  const int64_t kleft = o.k - kb0 * BK;
  TileLoader<TM, A_XC, Off> la;
  TileLoader<TM, B_XC, Off> lb;
  la.init(lda, m0, kb0 * BK);
  lb.init(ldb, n0, kb0 * BK);
  const int r0 = row0<TM>(), c0 = col0<TM>();
  float4 ra[TileLoader<TM, A_XC, Off>::NV], rb[TileLoader<TM, B_XC, Off>::NV];
  auto gload = [&](int kb) {
    const int kl = (int)min(kleft - (int64_t)kb * BK, (int64_t)BK);
    const bool chk = !interior || kl < BK;
    la.load(o.a, ra, lda, chk, ml, kl);
    lb.load(o.b, rb, ldb, chk, nl, kl);
    la.off += stepa;
    lb.off += stepb;
  };
  gload(0);
  la.store(As[0], ra);
  lb.store(Bs[0], rb);
  __syncthreads();
  for (int kb = 0; kb < nkb; ++kb) {
    const int buf = kb & 1;
    const bool more = kb + 1 < nkb;
    if (more) gload(kb + 1);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk * SA + r0]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk * SA + r0 + 32]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk * SB + c0]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk * SB + c0 + 16]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
      // column-outer order: measured faster than row-outer (fewer dispatch stalls)
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int i = 0; i < 8; ++i) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (more) {
      la.store(As[buf ^ 1], ra);
      lb.store(Bs[buf ^ 1], rb);
    }
    __syncthreads();
  }
}

// Layout chosen at run time (grouped kernels mix layouts in one launch).
template <int TM, typename Off>
__device__ __forceinline__ void ffma_unit_any(const Operands& o, int tm, int tn, int64_t kb0, int64_t kb1,
                                              float (&acc)[8][8], float* smem) {
  if (o.a_xc) {
    if (o.b_xc) ffma_unit_t<TM, true, true, Off>(o, tm, tn, kb0, kb1, acc, smem);
    else ffma_unit_t<TM, true, false, Off>(o, tm, tn, kb0, kb1, acc, smem);
  } else {
    if (o.b_xc) ffma_unit_t<TM, false, true, Off>(o, tm, tn, kb0, kb1, acc, smem);
    else ffma_unit_t<TM, false, false, Off>(o, tm, tn, kb0, kb1, acc, smem);
  }
}

template <int TM>
__device__ __forceinline__ int64_t row_of(int tm, int i) { return (int64_t)tm * TM + row_in_tile<TM>(i); }
template <int TM>
__device__ __forceinline__ int64_t col_of(int tn, int j) { return (int64_t)tn * TM + col_in_tile<TM>(j); }

// Asks L2 for the C tile's lines when a unit starts (beta != 0), so that the
// epilogue's loads of C hit L2: column-major C, TM columns of TM/32 128-byte
// lines (32 rows each), two lines per thread. Other layouts are left to the
// loads themselves.
template <int TM>
__device__ __forceinline__ void prefetch_c_tile(const Epi& e, int tm, int tn) {
  if (e.beta == 0.0f || e.rsc != 1) return;
  constexpr int LPC = TM / 32;  // lines per column
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int line = (int)threadIdx.x + u * Tile<TM>::THREADS;  // 0 .. TM*LPC-1
    const int64_t row = (int64_t)tm * TM + (line % LPC) * 32, col = (int64_t)tn * TM + (line / LPC);
    if (row < e.m && col < e.n) asm volatile("prefetch.global.L2 [%0];" ::"l"(e.c + row + col * e.csc));
  }
}

// C = beta*C + alpha*v for the eight outputs of register row i: all loads of
// C first, then the stores (one memory round trip per row, not per element).
template <int TM>
__device__ __forceinline__ void update_row(const Epi& e, int tm, int tn, int i, const float (&v)[8]) {
  const int64_t row = row_of<TM>(tm, i);
  float c0[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int64_t col = col_of<TM>(tn, j);
    c0[j] = (e.beta != 0.0f && row < e.m && col < e.n) ? e.c[row * e.rsc + col * e.csc] : 0.0f;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int64_t col = col_of<TM>(tn, j);
    if (row < e.m && col < e.n) {
      const float t = v[j] * e.alpha;
      e.c[row * e.rsc + col * e.csc] = (e.beta == 0.0f) ? t : fmaf(e.beta, c0[j], t);
    }
  }
}

// Epilogue; split-k partials ([splits][TM*TM] per tile, thread-interleaved)
// are summed by the last split in split order. Loads are issued a register
// row (8 values) at a time before any is used.
template <int TM>
__device__ __forceinline__ void ffma_finish(const Epi& e, float (&acc)[8][8], int tm, int tn, int splits, int sp,
                                            float* tile_partials, unsigned* counter, int* s_last) {
  constexpr int T = Tile<TM>::THREADS;
  const int tid = threadIdx.x;
  if (splits == 1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) update_row<TM>(e, tm, tn, i, acc[i]);
    return;
  }
  const size_t tile_elems = (size_t)TM * TM;
  float* part = tile_partials + (size_t)sp * tile_elems;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) part[(i * 8 + j) * T + tid] = acc[i][j];
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
    for (int i = 0; i < 8; ++i) {
      float v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) v[j] = __ldcg(tile_partials + (i * 8 + j) * T + tid);
      for (int q = 1; q < splits; ++q) {
        float w[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) w[j] = __ldcg(tile_partials + (size_t)q * tile_elems + (i * 8 + j) * T + tid);
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] += w[j];
      }
      update_row<TM>(e, tm, tn, i, v);
    }
    if (tid == 0) *counter = 0u;
  }
  __syncthreads();
}

}  // namespace ffma
}  // namespace momms
