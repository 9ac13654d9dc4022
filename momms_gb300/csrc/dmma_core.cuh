// Building blocks of the FP64 DMMA GEMM kernels (single-problem and grouped):
// TMA staging of 128B-swizzled A/B tiles, the warp-level DMMA k loop, and the
// epilogue with optional split-k fix-up.
//
// CTA tile 128 x 128, k-blocks of 16, a 4-stage shared-memory ring; one TMA
// producer warp and eight DMMA warps (warp tile 64 x 32 = 8 x 4 blocks of
// 8 x 8). An operand whose non-k index is contiguous ("x-contiguous":
// column-major A, row-major B) is staged as 16-wide sub-tiles [BK][16];
// a k-contiguous one as [128][BK]. Both use the 128-byte swizzle.
#pragma once
#include "common.cuh"

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

// Output description for the epilogue.
struct Epi {
  int64_t m, n;
  double alpha, beta;
  double* c;
  int64_t rsc, csc;
};

__device__ __forceinline__ void store_c(const Epi& e, int64_t row, int64_t col, double v) {
  if (row < e.m && col < e.n) {
    double* cp = e.c + row * e.rsc + col * e.csc;
    double s = v * e.alpha;
    *cp = (e.beta == 0.0) ? s : fma(e.beta, *cp, s);
  }
}

// Producer: TMA loads of k-blocks [kb0, kb1) of output tile (tm, tn).
// Returns false if a bounded wait expired.
__device__ __forceinline__ bool produce_unit(const CUtensorMap* tmA, const CUtensorMap* tmB, bool a_xc, bool b_xc,
                                             int tm, int tn, int64_t kb0, int64_t kb1, uint8_t* sA, uint8_t* sB,
                                             uint64_t* full, uint64_t* empty, int& stage, uint32_t& phase,
                                             unsigned* status) {
  for (int64_t kb = kb0; kb < kb1; ++kb) {
    if (!mbar_wait_bounded(&empty[stage], phase ^ 1)) {
      report_status(status, DEV_TIMEOUT_EMPTY);
      return false;
    }
    mbar_arrive_expect_tx(&full[stage], A_STAGE + B_STAGE);
    uint8_t* a_dst = sA + stage * A_STAGE;
    uint8_t* b_dst = sB + stage * B_STAGE;
    const int32_t kc = (int32_t)(kb * BK);
    if (a_xc) {
#pragma unroll
      for (int j = 0; j < BM / 16; ++j) tma_load_2d(a_dst + j * SUB, tmA, &full[stage], tm * BM + 16 * j, kc);
    } else {
      tma_load_2d(a_dst, tmA, &full[stage], kc, tm * BM);
    }
    if (b_xc) {
#pragma unroll
      for (int j = 0; j < BN / 16; ++j) tma_load_2d(b_dst + j * SUB, tmB, &full[stage], tn * BN + 16 * j, kc);
    } else {
      tma_load_2d(b_dst, tmB, &full[stage], kc, tn * BN);
    }
    if (++stage == STAGES) {
      stage = 0;
      phase ^= 1;
    }
  }
  return true;
}

// Bit (i*4 + j) is set when the warp's 8x8 block (i, j) holds an element of
// the m x n output; blocks entirely outside are not multiplied (TMA fills
// them with zeros), so edge tiles and small problems spend FP64 work only on
// live blocks. Warp-uniform.
__device__ __forceinline__ uint32_t live_mask(int64_t row_base, int64_t col_base, int64_t m, int64_t n) {
  uint32_t mask = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (row_base + i * 8 < m && col_base + j * 8 < n) mask |= 1u << (i * 4 + j);
  return mask;
}

// Consumer: accumulate k-blocks [kb0, kb1) of the current unit into acc.
// Returns false if a bounded wait expired.
__device__ __forceinline__ bool consume_unit(bool a_xc, bool b_xc, int64_t kb0, int64_t kb1, uint32_t live,
                                             const uint8_t* sA, const uint8_t* sB, uint64_t* full, uint64_t* empty,
                                             int& stage, uint32_t& phase, int wm, int wn, int lane,
                                             double (&acc)[8][4][2], unsigned* status) {
  for (int64_t kb = kb0; kb < kb1; ++kb) {
    if (!mbar_wait_bounded(&full[stage], phase)) {
      report_status(status, DEV_TIMEOUT_FULL);
      return false;
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
        af[i] = *reinterpret_cast<const double*>(a + (a_xc ? off_xc(r, kk) : off_kc(r, kk)));
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int cidx = wn * 32 + j * 8 + (lane >> 2);
        bf[j] = *reinterpret_cast<const double*>(b + (b_xc ? off_xc(cidx, kk) : off_kc(cidx, kk)));
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (live & (1u << (i * 4 + j))) dmma(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[stage]);
    if (++stage == STAGES) {
      stage = 0;
      phase ^= 1;
    }
  }
  return true;
}

// Epilogue of one unit. With splits == 1 the tile goes straight to C.
// Otherwise this split's partial tile is published in `tile_partials`
// ([splits][BM*BN], thread-interleaved), and the last split to arrive on
// `counter` sums all partials in split order 0..splits-1 (a fixed order: the
// result does not depend on which CTA finishes last), writes C and resets
// the counter to zero.
//
// A thread's 64 outputs are handled in groups of EPI_ROWS 8-row blocks (8
// outputs each): every load of a group (C for beta != 0, the partials of one
// split) is issued before the first value is used, so a group costs one
// memory round trip per pass instead of one per element.
constexpr int EPI_ROWS = 1;
__device__ __forceinline__ void finish_unit(const Epi& e, double (&acc)[8][4][2], int64_t row0, int64_t col0,
                                            int splits, int sp, double* tile_partials, unsigned* counter, int ctid,
                                            int* s_last) {
  constexpr int G = EPI_ROWS;
  const size_t tile_elems = (size_t)BM * BN;
  // element (i, j, q) of this thread: row row0 + 8i, column col0 + 8j + q
  auto live = [&](int i, int j, int q) { return row0 + i * 8 < e.m && col0 + j * 8 + q < e.n; };
  auto cptr = [&](int i, int j, int q) { return e.c + (row0 + i * 8) * e.rsc + (col0 + j * 8 + q) * e.csc; };
  auto slot = [&](int i, int j, int q) { return ((i * 4 + j) * 2 + q) * CONSUMERS + ctid; };
  // C = beta*C + alpha*v for block rows g*G .. g*G+G-1
  auto update_group = [&](int g, const double (&v)[G][4][2]) {
    double c0[G][4][2];
#pragma unroll
    for (int ii = 0; ii < G; ++ii)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 2; ++q)
          c0[ii][j][q] = (e.beta != 0.0 && live(g * G + ii, j, q)) ? *cptr(g * G + ii, j, q) : 0.0;
#pragma unroll
    for (int ii = 0; ii < G; ++ii)
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 2; ++q)
          if (live(g * G + ii, j, q)) {
            const double t = v[ii][j][q] * e.alpha;
            *cptr(g * G + ii, j, q) = (e.beta == 0.0) ? t : fma(e.beta, c0[ii][j][q], t);
          }
  };
  if (splits == 1) {
#pragma unroll
    for (int g = 0; g < 8 / G; ++g) {
      double v[G][4][2];
#pragma unroll
      for (int ii = 0; ii < G; ++ii)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q = 0; q < 2; ++q) v[ii][j][q] = acc[g * G + ii][j][q];
      update_group(g, v);
    }
    return;
  }
  // Partials exist only for the tile's entries inside C: a small problem's
  // mostly-empty tile writes and re-reads just its live part.
  double* part = tile_partials + (size_t)sp * tile_elems;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 2; ++q)
        if (live(i, j, q)) part[slot(i, j, q)] = acc[i][j][q];
  __threadfence();
  consumer_sync();
  if (ctid == 0) {
    unsigned prev = atomicAdd(counter, 1u);
    *s_last = (prev == (unsigned)(splits - 1)) ? 1 : 0;
  }
  consumer_sync();
  if (*s_last) {
    __threadfence();
#pragma unroll
    for (int g = 0; g < 8 / G; ++g) {
      double v[G][4][2];
#pragma unroll
      for (int ii = 0; ii < G; ++ii)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
          for (int q = 0; q < 2; ++q)
            v[ii][j][q] = live(g * G + ii, j, q) ? __ldcg(tile_partials + slot(g * G + ii, j, q)) : 0.0;
      for (int t = 1; t < splits; ++t) {
        const double* pt = tile_partials + (size_t)t * tile_elems;
        double w[G][4][2];
#pragma unroll
        for (int ii = 0; ii < G; ++ii)
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 2; ++q) w[ii][j][q] = live(g * G + ii, j, q) ? __ldcg(pt + slot(g * G + ii, j, q)) : 0.0;
#pragma unroll
        for (int ii = 0; ii < G; ++ii)
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int q = 0; q < 2; ++q) v[ii][j][q] += w[ii][j][q];
      }
      update_group(g, v);
    }
    if (ctid == 0) *counter = 0u;
  }
  consumer_sync();
}

// Shared-memory carve-up and barrier initialisation common to the kernels.
struct Smem {
  uint8_t* sA;
  uint8_t* sB;
  uint64_t* full;
  uint64_t* empty;
  int* s_last;
};

__device__ __forceinline__ Smem setup_smem(uint8_t* smem_raw) {
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  Smem s;
  s.sA = smem;
  s.sB = smem + STAGES * A_STAGE;
  s.full = reinterpret_cast<uint64_t*>(s.sB + STAGES * B_STAGE);
  s.empty = s.full + STAGES;
  s.s_last = reinterpret_cast<int*>(s.empty + STAGES);
  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&s.full[i], 1);
      mbar_init(&s.empty[i], CONSUMER_WARPS);
    }
    fence_barrier_init();
  }
  __syncthreads();
  return s;
}

}  // namespace dmma
}  // namespace momms
