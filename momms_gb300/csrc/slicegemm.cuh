// The slice-pair GEMM engine on tcgen05: C-tile accumulation of sums of
// products of operand "planes" (precision slices of A and B) through TMEM.
//
//   for each output tile (persistent, one CTA per SM, 128 x 256 tiles):
//     for each group g (processed in order):
//       S_g = sum over pairs (a, b) in g of  A_plane[a] * B_plane[b]^T
//       accumulated in TMEM in chunks (runs of (pair, k-block) steps within a
//       bound, Params::pair_w); each finished chunk is handed to the
//       epilogue (ping-pong TMEM buffers)
//
// Planes are K-major in HBM ([plane][row][k], k contiguous) and are loaded by
// TMA as 128-byte-wide k-blocks with the 128B swizzle that the tcgen05 shared
// memory descriptors expect. Warp roles: warp 0 issues TMA, warp 1 (one
// thread) issues tcgen05.mma and commits, warps 2..9 drain TMEM.
//
// Three epilogues:
//   EPI_F32   : one group; finished chunks are summed in FP32 registers
//               (round to nearest) and C = alpha*sum + beta*C is written at
//               the end of the tile. Used by the split-TF32 f32 path (pairs
//               lo*hi, hi*lo, hi*hi).
//   EPI_OZAKI : integer-valued slices; every chunk is exact in FP32 (the
//               host sizes chunks so that sums of absolute products stay
//               within 2^24) and is converted and added into int32
//               accumulators; at the end of each group the
//               exact sums are written to that group's int32 plane (the FP64
//               recombination runs afterwards in its own kernel, so no FP64
//               work sits in this pipeline).
//   EPI_BOUND : one group of one pair, bf16 magnitude planes |a| 2^-e_i and
//               |b| 2^-f_j rounded toward zero: the FP32 sum is a lower bound
//               L_ij of (|A||B|)_ij 2^-(e_i+f_j) (after a factor for the
//               accumulation's rounding). Nothing is stored per entry: each
//               tile reduces the worst-case error ratios
//                 q1 = (sum_p |a_ip| 2^-e_i + sum_p |b_pj| 2^-f_j) / L_ij,
//                 q2 = k / L_ij
//               (upward-rounded) to two maxima posted with atomicMax, and
//               counts the entries with L_ij = 0; from these the host picks a
//               slice count that holds for every entry. With count_only the
//               planes are 0/1 indicators of nonzero elements and only the
//               entries with a nonzero sum are counted.
#pragma once
#include <stdlib.h>

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <vector>

#include "tc_common.cuh"

namespace momms {
namespace sp {

// A stage holds one k-block of each operand: 128 bytes of k per row (64 fp16
// or 32 fp32 elements) in the 128-byte swizzle. (64-byte k-blocks with the
// 64-byte swizzle fit nine stages instead of four but measured 25 % slower:
// twice the TMA row requests per byte.)
constexpr int BM = 128, BN = 256, STAGES = 4;
constexpr int ROW_BYTES = 128;
constexpr int KSTEPS = ROW_BYTES / 32;  // MMAs per stage (each consumes 32 bytes of k)
constexpr int A_TILE = BM * ROW_BYTES;
constexpr int B_TILE = BN * ROW_BYTES;
constexpr int STAGE_BYTES = A_TILE + B_TILE;  // 48 KB
constexpr int EPI_WARPS = 8;                     // 2 per TMEM lane quarter
constexpr int EPI_COLS = BN / (EPI_WARPS / 4);   // columns drained per thread
constexpr int THREADS = (2 + EPI_WARPS) * 32;
constexpr int TMEM_COLS = 512;  // two 128 x 256 f32 accumulators
constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + 256;
constexpr int MAX_GROUPS = 160, MAX_PAIRS = 160;

enum { EPI_F32 = 0, EPI_OZAKI = 1, EPI_BOUND = 2 };

struct Params {
  int64_t m, n;
  int kblocks;  // k-blocks per plane
  int kelems;   // elements per k-block (64 for f16, 32 for tf32: 128 bytes)
  int tiles_m, tiles_n;
  int ngroups;
  int gchunk;  // groups per work unit: a tile's groups may run as separate units (0 = all)
  int group_begin[MAX_GROUPS + 1];
  // TMEM accumulation chunks: a chunk is a run of consecutive (pair, k-block)
  // steps of one group whose weights pair_w sum to at most chunk_cap; with
  // merge_pairs a chunk continues from one pair into the next (the Ozaki
  // path, whose chunk sums are exact, so chunking never changes a result),
  // otherwise every pair starts a new chunk. group_chunks[g]: chunks of
  // group g (plan_chunks).
  int pair_w[MAX_PAIRS];
  int chunk_cap, merge_pairs;
  int group_chunks[MAX_GROUPS];
  uint8_t pair_a[MAX_PAIRS], pair_b[MAX_PAIRS];
  // EPI_F32
  float alpha_f, beta_f;
  float* c32;
  // EPI_OZAKI: exact group sums, one int32 plane per group, tile-blocked:
  // element (row, col) at (col / BN) * (tiles_m * BM * BN) + (row / BM) * BM * BN
  // + (col % BN) * BM + row % BM, so that each CTA tile is written as one
  // contiguous block
  int* sbuf;
  int64_t plane;
  int64_t rsc, csc;
  // EPI_BOUND: row sums of the scaled magnitudes of A (m) and B's columns
  // (n) in units of 2^-40, each term rounded up; the lower-bound factor for
  // the accumulation; k; the two maxima (bit patterns of non-negative floats)
  const unsigned long long* msum_a;
  const unsigned long long* msum_b;
  float lb_scale, kf;
  unsigned* bound_out;                // [0], [1]: the maxima
  unsigned long long* bound_count;  // entries counted
  int count_only;
  int64_t unit_begin;  // grouped launches: this problem's first work unit
  unsigned* status;
};

// A grouped launch of the CTA-pair kernel: many problems, each with its own
// Params (schedule, sizes, output) and tensor maps, in device memory. Work
// unit u belongs to the last problem whose unit_begin <= u.
struct GroupTable {
  const Params* probs;      // sorted by unit_begin
  const CUtensorMap* maps;  // [2 * nprobs]: each problem's A map and B half-tile map (64-byte aligned)
  int nprobs;
  int64_t units;
};

__device__ __forceinline__ bool aborted(volatile int* flag) { return *flag != 0; }

// Output tile of work item t: groups of 16 m-tiles swept n-tile by n-tile,
// so that the ~152 tiles in flight at once share 16 A row panels and about
// 10 B column panels of each slice plane in L2 (a plain column-major sweep
// would touch a whole 128 MB plane per pair at m = 8192).
template <int G>
__device__ __forceinline__ void tile_coords(int64_t t, int tiles_m, int tiles_n, int& tm, int& tn) {
  const int64_t per_group = (int64_t)G * tiles_n;
  const int64_t g = t / per_group, r = t % per_group;
  const int first = (int)(g * G);
  const int gm = min(G, tiles_m - first);
  tm = first + (int)(r % gm);
  tn = (int)(r / gm);
}

// Accumulators of drained chunks: Ozaki sums are int32 (each chunk value is
// an integer of magnitude <= 2^24, exact in FP32, converted exactly);
// split-TF32 sums are FP32.
template <int EPI>
using EpiAcc = typename std::conditional<EPI == EPI_OZAKI, int, float>::type;

// Drains one TMEM chunk (this thread's row, NC columns from taddr) into S.
// The loads run one 16-column batch ahead of the adds: a batch's wait comes
// after the previous batch's adds.
template <int EPI, int NC>
__device__ __forceinline__ void drain_chunk(uint32_t taddr, EpiAcc<EPI> (&S)[NC]) {
  uint32_t ra[16], rb[16];
  tc::ld16(taddr, ra);
#pragma unroll
  for (int pc = 0; pc < NC / 16; ++pc) {
    uint32_t(&cur)[16] = (pc & 1) ? rb : ra;
    uint32_t(&nxt)[16] = (pc & 1) ? ra : rb;
    tc::ld_wait(cur);
    if (pc + 1 < NC / 16) tc::ld16(taddr + (pc + 1) * 16, nxt);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (EPI == EPI_OZAKI) S[pc * 16 + j] += __float2int_rz(__uint_as_float(cur[j]));
      else S[pc * 16 + j] += __uint_as_float(cur[j]);
    }
  }
}

// EPI_BOUND: this thread's row against its NC columns, reduced over the warp
// and posted to the two maxima. Every lane calls it (rows past m contribute 0).
template <int NC>
__device__ __forceinline__ void bound_tile(const Params& p, int64_t row, int64_t col0, const float (&S)[NC]) {
  static_assert(NC % 32 == 0, "columns are shared out 32 per lane round");
  float m1 = 0.0f, m2 = 0.0f;
  unsigned cnt = 0;
  // columns of this tile inside C (the same for the whole warp)
  const int nvalid = (int)min((int64_t)NC, max((int64_t)0, p.n - col0));
  if (p.count_only) {
    if (row < p.m) {
#pragma unroll
      for (int j = 0; j < NC; ++j) cnt += (j < nvalid && S[j] > 0.0f) ? 1u : 0u;
    }
  } else {
    // The warp's 32 rows share their NC columns: each lane converts the
    // column sums of every 32nd column once (upward, units of 2^-40) and the
    // entries take them by shuffle.
    const int lane = threadIdx.x & 31;
    float sbl[NC / 32];
#pragma unroll
    for (int q = 0; q < NC / 32; ++q)
      sbl[q] = 32 * q + lane < nvalid ? __fmul_ru(__ull2float_ru(p.msum_b[col0 + 32 * q + lane]), 0x1p-40f) : 0.0f;
    const bool rv = row < p.m;
    const float sa = rv ? __fmul_ru(__ull2float_ru(p.msum_a[row]), 0x1p-40f) : 0.0f;
    // q2 = k / L needs only the row's smallest L: one reciprocal per row.
    // q1 = (sa + sb) / L: an entry whose (sa + sb), rounded up, is at most
    // m1 * L rounded down cannot raise m1 (its quotient is at most m1), so
    // the upward quotient is formed only for the others.
    float lmin = INFINITY;
#pragma unroll
    for (int j = 0; j < NC; ++j) {
      const float sb = __shfl_sync(0xffffffffu, sbl[j >> 5], j & 31);
      const float lb = __fmul_rd(S[j], p.lb_scale);
      // L = 0: no p with both a_ip and b_pj nonzero (the entry has no
      // error), or every term below FP32's range: counted, the host tells
      // the two apart
      if (rv && j < nvalid) {
        if (lb > 0.0f) {
          const float x = __fadd_ru(sa, sb);
          if (x > __fmul_rd(m1, lb)) m1 = fmaxf(m1, __fmul_ru(x, __frcp_ru(lb)));
          lmin = fminf(lmin, lb);
        } else {
          ++cnt;
        }
      }
    }
    if (lmin < INFINITY) m2 = __fmul_ru(p.kf, __frcp_ru(lmin));  // >= k / L for every entry of the row
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    // Non-negative floats order like their bit patterns. Every warp of every
    // tile reports here: the maxima only grow, so a warp below the value
    // already posted skips its atomic (same-address atomics serialise in L2;
    // at 8192 x 8192 x 64 they cost most of the kernel).
    if (!p.count_only) {
      const volatile unsigned* cur = p.bound_out;
      if (__float_as_uint(m1) > cur[0]) atomicMax(&p.bound_out[0], __float_as_uint(m1));
      if (__float_as_uint(m2) > cur[1]) atomicMax(&p.bound_out[1], __float_as_uint(m2));
    }
    if (cnt) atomicAdd(p.bound_count, (unsigned long long)cnt);
  }
}

// Split-TF32 epilogue: asks L2 for the C lines this thread's warp will
// read at the end of the tile (beta != 0), issued when the tile starts, so
// that the epilogue's loads of C hit L2 instead of HBM. Column-major C: a
// warp's 32 rows of one column are one 128-byte line, so lane L takes the
// columns L, L + 32, ... of the thread's EPI_COLS; other layouts are left to
// the loads themselves.
template <int NC>
__device__ __forceinline__ void prefetch_c_rows(const Params& p, int64_t row_of_lane0, int64_t col0, int lane) {
  if (p.beta_f == 0.0f || p.rsc != 1 || row_of_lane0 >= p.m) return;
  const float* base = p.c32 + row_of_lane0;
#pragma unroll
  for (int j = lane; j < NC; j += 32) {
    const int64_t col = col0 + j;
    if (col < p.n) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + col * p.csc));
  }
}

template <int KIND, int EPI>
__global__ void __launch_bounds__(THREADS, 1)
    slice_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ Params p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* tfull = empty + STAGES;  // [2]
  uint64_t* tempty = tfull + 2;      // [2]
  uint64_t* drain = tempty + 2;      // used only when aborting
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // work units: output tiles (times group chunks), one CTA each
  const int64_t unit0 = (int64_t)blockIdx.x;
  const int64_t unit_step = (int64_t)gridDim.x;
  const int units_m = p.tiles_m;
  // work unit t: tile (pair) t % tile_units, groups [g_begin(t), g_end(t)) -
  // group-major, so that units in flight read the same digit planes
  const int64_t tile_units = (int64_t)units_m * p.tiles_n;
  const int gchunk = p.gchunk > 0 ? p.gchunk : p.ngroups;
  const int64_t units = tile_units * ceil_div_dev(p.ngroups, gchunk);
  auto g_begin = [&](int64_t t) { return (int)(t / tile_units) * gchunk; };
  auto g_end = [&](int64_t t) { return min(p.ngroups, g_begin(t) + gchunk); };
  // round r hands units [r*step, (r+1)*step) to the CTAs (clusters), in
  // reverse order on odd rounds: units are ordered by falling cost (largest
  // groups first), so this snake order evens out the per-CTA totals
  auto unit_at = [&](int64_t r) {
    return r * unit_step + ((r & 1) ? (unit_step - 1 - unit0) : unit0);
  };
  auto coords = [&](int64_t t, int& tm, int& tn) { tile_coords<16>(t, units_m, p.tiles_n, tm, tn); };

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], EPI_WARPS);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_slot, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------ TMA producer ------------------------------
    if (lane == 0) {
      prefetch_tensormap(&tmA);
      prefetch_tensormap(&tmB);
      int stage = 0;
      uint32_t ph = 0;
      uint32_t armed = 0;  // bit s: stage s has been armed at least once
      uint32_t last_ph = 0;  // bit s: parity of the phase last armed on stage s
      for (int64_t r = 0; r * unit_step < units && !aborted(abort_flag); ++r) {
        const int64_t t = unit_at(r);
        if (t >= units) continue;
        int tm, tn;
        coords(t % tile_units, tm, tn);
        for (int g = g_begin(t); g < g_end(t); ++g) {
          for (int pi = p.group_begin[g]; pi < p.group_begin[g + 1]; ++pi) {
            for (int kb = 0; kb < p.kblocks; ++kb) {
              if (!mbar_wait_bounded(&empty[stage], ph ^ 1)) {
                report_status(p.status, DEV_TIMEOUT_EMPTY);
                *abort_flag = 1;
                // let every copy already issued land before the CTA exits
                for (int s = 0; s < STAGES; ++s)
                  if ((armed >> s) & 1u) mbar_wait_bounded(&full[s], (last_ph >> s) & 1u);
                goto producer_done;
              }
              armed |= 1u << stage;
              last_ph = (last_ph & ~(1u << stage)) | (ph << stage);
              mbar_arrive_expect_tx(&full[stage], STAGE_BYTES);
              uint8_t* sa = smem + stage * STAGE_BYTES;
              tma_load_3d(sa, &tmA, &full[stage], kb * p.kelems, tm * BM, p.pair_a[pi]);
              tma_load_3d(sa + A_TILE, &tmB, &full[stage], kb * p.kelems, tn * BN, p.pair_b[pi]);
              if (++stage == STAGES) {
                stage = 0;
                ph ^= 1;
              }
            }
          }
        }
      }
    producer_done:;
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer ------------------------------
    if (lane == 0) {
      const uint32_t idv = tc::idesc(tc::kind_fmt(KIND), BM, BN);
      int stage = 0;
      uint32_t ph = 0;
      int buf = 0;
      uint32_t acc_ph[2] = {0, 0};
      for (int64_t r = 0; r * unit_step < units && !aborted(abort_flag); ++r) {
        const int64_t t = unit_at(r);
        if (t >= units) continue;
        for (int g = g_begin(t); g < g_end(t); ++g) {
          int load = 0;
          bool open = false;
          uint32_t d_tmem = 0;
          for (int pp = p.group_begin[g]; pp < p.group_begin[g + 1]; ++pp) {
            const int w = p.pair_w[pp];
            if (open && !p.merge_pairs) {
              tc::commit(&tfull[buf]);
              acc_ph[buf] ^= 1;
              buf ^= 1;
              open = false;
            }
            for (int st = 0; st < p.kblocks;) {
              if (open && load + w > p.chunk_cap) {
                tc::commit(&tfull[buf]);
                acc_ph[buf] ^= 1;
                buf ^= 1;
                open = false;
              }
              bool fresh = false;
              if (!open) {
                if (!mbar_wait_bounded(&tempty[buf], acc_ph[buf] ^ 1)) {
                  report_status(p.status, DEV_TIMEOUT_TMEM);
                  *abort_flag = 1;
                  goto mma_done;
                }
                tc::fence_after();
                d_tmem = tmem_base + (uint32_t)(buf * BN);
                load = 0;
                open = fresh = true;
              }
              // the k-blocks of this pair that still fit in the open chunk
              const int s0 = st, s1 = min(p.kblocks, st + (p.chunk_cap - load) / w);
              for (; st < s1; ++st) {
                if (!mbar_wait_bounded(&full[stage], ph)) {
                  report_status(p.status, DEV_TIMEOUT_FULL);
                  *abort_flag = 1;
                  goto mma_done;
                }
                tc::fence_after();
                const uint32_t a_addr = smem_u32(smem + stage * STAGE_BYTES);
                const uint32_t b_addr = a_addr + A_TILE;
#pragma unroll
                for (int kk = 0; kk < KSTEPS; ++kk)
                  tc::mma<KIND>(d_tmem, tc::sdesc_k128(a_addr + kk * 32), tc::sdesc_k128(b_addr + kk * 32), idv,
                                (fresh && st == s0 && kk == 0) ? 0u : 1u);
                tc::commit(&empty[stage]);
                if (++stage == STAGES) {
                  stage = 0;
                  ph ^= 1;
                }
              }
              load += (s1 - s0) * w;
            }
          }
          if (open) {
            tc::commit(&tfull[buf]);
            acc_ph[buf] ^= 1;
            buf ^= 1;
          }
        }
      }
    mma_done:
      if (aborted(abort_flag)) {
        // wait (bounded) until every MMA issued so far has completed, so that
        // TMEM is not released under a running MMA
        tc::commit(drain);
        mbar_wait_bounded(drain, 0);
      }
    }
  } else {
    // ------------------------------ epilogue ------------------------------
    const int q = warp & 3;              // TMEM lane quarter this warp may access
    const int h = (warp - 2) >> 2;       // column group: cols h*EPI_COLS .. +EPI_COLS-1
    const int r_local = q * 32 + lane;
    int buf = 0;
    uint32_t acc_ph[2] = {0, 0};
    for (int64_t r = 0; r * unit_step < units && !aborted(abort_flag); ++r) {
      const int64_t t = unit_at(r);
      if (t >= units) continue;
      int tm, tn;
      coords(t % tile_units, tm, tn);
      const int64_t row = (int64_t)tm * BM + r_local;
      const int64_t col0 = (int64_t)tn * BN + h * EPI_COLS;
      if (EPI == EPI_F32) prefetch_c_rows<EPI_COLS>(p, (int64_t)tm * BM + q * 32, col0, lane);
      // per-thread accumulators of finished chunks: exact int32 digit sums
      // (Ozaki) or FP32 sums rounded to nearest (split-TF32), which keeps the
      // tensor core's internal accumulation to one chunk at a time
      EpiAcc<EPI> S[EPI_COLS];
#pragma unroll
      for (int j = 0; j < EPI_COLS; ++j) S[j] = EpiAcc<EPI>(0);
      for (int g = g_begin(t); g < g_end(t); ++g) {
        for (int c = 0; c < p.group_chunks[g]; ++c) {
          if (!mbar_wait_bounded(&tfull[buf], acc_ph[buf])) {
            report_status(p.status, DEV_TIMEOUT_MMA);
            *abort_flag = 1;
            goto epi_done;
          }
          tc::fence_after();
          const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN + h * EPI_COLS);
          drain_chunk<EPI, EPI_COLS>(taddr, S);
          tc::fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&tempty[buf]);
          acc_ph[buf] ^= 1;
          buf ^= 1;
        }
        if (EPI == EPI_OZAKI) {
          // end of group g: publish the exact int32 sums (column-major plane g)
          if (row < p.m) {
            // tile-blocked plane: this CTA's 128 x 256 tile is one contiguous
            // block, column after column of 128 rows (see the host's plane layout)
            int* srow = p.sbuf + (size_t)g * p.plane + (size_t)tn * ((size_t)p.tiles_m * BM * BN) +
                        (size_t)tm * (BM * BN) + (size_t)(h * EPI_COLS) * BM + r_local;
#pragma unroll
            for (int j = 0; j < EPI_COLS; ++j) {
              const int64_t col = col0 + j;
              if (col < p.n) srow[j * BM] = S[j];
            }
          }
#pragma unroll
          for (int j = 0; j < EPI_COLS; ++j) S[j] = EpiAcc<EPI>(0);
        }
      }
      if constexpr (EPI == EPI_BOUND) bound_tile<EPI_COLS>(p, row, col0, S);
      if (EPI == EPI_F32 && row < p.m) {
        // C is read 8 columns at a time, every load of a group issued before
        // the first use (one memory round trip per group, not per element)
        float* crow = p.c32 + row * p.rsc;
#pragma unroll
        for (int j0 = 0; j0 < EPI_COLS; j0 += 8) {
          float c0[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t col = col0 + j0 + j;
            c0[j] = (p.beta_f != 0.0f && col < p.n) ? crow[col * p.csc] : 0.0f;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t col = col0 + j0 + j;
            if (col < p.n) {
              const float v = (float)S[j0 + j] * p.alpha_f;
              crow[col * p.csc] = (p.beta_f == 0.0f) ? v : fmaf(p.beta_f, c0[j], v);
            }
          }
        }
      }
    }
  epi_done:;
  }

  // reconverge each warp (its lane 0 may have run a role loop alone) before
  // the CTA-wide barrier, which requires whole warps
  __syncwarp();
  tc::fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// CTA-pair kernel (cta_group::2). A cluster of two CTAs computes a 256 x 256
// output tile with one MMA stream: each CTA holds 128 rows of A and 128 rows
// (columns of the output) of B per stage, and the even CTA issues
// tcgen05.mma.cta_group::2, which reads both CTAs' shared memory and writes
// 128 output rows into each CTA's TMEM. Against the single-CTA kernel this
// reads two thirds of the shared-memory bytes per FLOP (the B half is read
// once for both SMs) and a stage is 32 KB, so seven stages fit.
//   full[s]   (even CTA)  both CTAs' TMA loads complete here (64 KB)
//   empty[s]  (each CTA)  the even CTA's commit, multicast: stage s is free
//   tfull[b]  (each CTA)  the even CTA's commit, multicast: accumulator b done
//   tempty[b] (even CTA)  all 16 epilogue warps of the pair: b drained
// ---------------------------------------------------------------------------
constexpr int PSTAGES = 7;
constexpr int P_STAGE_BYTES = A_TILE + B_TILE / 2;  // 32 KB
constexpr int P_SMEM_BYTES = 1024 + PSTAGES * P_STAGE_BYTES + 256;

template <int KIND, int EPI, bool GROUPED = false>
__global__ void __launch_bounds__(THREADS, 1)
    slice_gemm_pair_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmBh,
                           const __grid_constant__ Params p, const __grid_constant__ GroupTable gt) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + PSTAGES * P_STAGE_BYTES);
  uint64_t* empty = full + PSTAGES;
  uint64_t* tfull = empty + PSTAGES;  // [2]
  uint64_t* tempty = tfull + 2;       // [2]
  uint64_t* drain = tempty + 2;       // used only when aborting
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();
  const bool leader = (rank == 0);
  const int64_t unit0 = (int64_t)cluster_id_x(), unit_step = (int64_t)cluster_count_x();
  // A problem's work units: vertical tile pairs x chunks of its groups,
  // group-major (units in flight read the same digit planes).
  auto tile_units_of = [](const Params& P) { return (int64_t)((P.tiles_m + 1) / 2) * P.tiles_n; };
  auto gchunk_of = [](const Params& P) { return P.gchunk > 0 ? P.gchunk : P.ngroups; };
  const int64_t units = GROUPED ? gt.units : tile_units_of(p) * ceil_div_dev(p.ngroups, gchunk_of(p));
  unsigned* status = GROUPED ? gt.probs[0].status : p.status;
  // round r hands units [r*step, (r+1)*step) to the CTAs (clusters), in
  // reverse order on odd rounds: units are ordered by falling cost (largest
  // groups first), so this snake order evens out the per-CTA totals
  auto unit_at = [&](int64_t r) {
    return r * unit_step + ((r & 1) ? (unit_step - 1 - unit0) : unit0);
  };
  // Calls fn(problem, its A map, its B map, unit within the problem).
  auto with_unit = [&](int64_t u, auto&& fn) -> bool {
    if constexpr (GROUPED) {
      int lo = 0, hi = gt.nprobs - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (gt.probs[mid].unit_begin <= u) lo = mid;
        else hi = mid - 1;
      }
      const Params& P = gt.probs[lo];
      return fn(P, &gt.maps[2 * lo], &gt.maps[2 * lo + 1], u - P.unit_begin);
    } else {
      return fn(p, &tmA, &tmBh, u);
    }
  };
  // tile of unit t of problem P (rank 1 of an odd last pair reads zero rows, writes nothing)
  auto coords = [&](const Params& P, int64_t t, int& tm, int& tn) {
    int um;
    tile_coords<8>(t % tile_units_of(P), (P.tiles_m + 1) / 2, P.tiles_n, um, tn);
    tm = 2 * um + (int)rank;
  };
  auto groups_of = [&](const Params& P, int64_t t, int& g0, int& g1) {
    const int gc = gchunk_of(P);
    g0 = (int)(t / tile_units_of(P)) * gc;
    g1 = min(P.ngroups, g0 + gc);
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < PSTAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 2 * EPI_WARPS);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc2(tmem_slot, TMEM_COLS);
    tc::tmem_relinquish2();
  }
  tc::fence_before();
  __syncthreads();
  cluster_sync();  // the pair's barriers exist before any remote arrival
  tc::fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------ TMA producer (both CTAs) ------------------------------
    if (lane == 0) {
      if (!GROUPED) {
        prefetch_tensormap(&tmA);
        prefetch_tensormap(&tmBh);
      }
      int stage = 0;
      uint32_t ph = 0;
      auto produce = [&](const Params& P, const CUtensorMap* mA, const CUtensorMap* mB, int64_t t) -> bool {
        int tm, tn, g0, g1;
        coords(P, t, tm, tn);
        groups_of(P, t, g0, g1);
        for (int g = g0; g < g1; ++g) {
          for (int pi = P.group_begin[g]; pi < P.group_begin[g + 1]; ++pi) {
            for (int kb = 0; kb < P.kblocks; ++kb) {
              if (!mbar_wait_bounded(&empty[stage], ph ^ 1)) {
                report_status(status, DEV_TIMEOUT_EMPTY);
                *abort_flag = 1;
                return false;
              }
              if (leader) mbar_arrive_expect_tx(&full[stage], 2 * P_STAGE_BYTES);
              uint8_t* sa = smem + stage * P_STAGE_BYTES;
              const uint32_t bar = mapa_shared(&full[stage], 0);
              tma_load_3d_pair(sa, mA, bar, kb * P.kelems, tm * BM, P.pair_a[pi]);
              tma_load_3d_pair(sa + A_TILE, mB, bar, kb * P.kelems, tn * BN + (int)rank * (BN / 2), P.pair_b[pi]);
              if (++stage == PSTAGES) {
                stage = 0;
                ph ^= 1;
              }
            }
          }
        }
        return true;
      };
      bool ok = true;
      for (int64_t r = 0; r * unit_step < units && ok && !aborted(abort_flag); ++r) {
        const int64_t u = unit_at(r);
        if (u >= units) continue;
        ok = with_unit(u, produce);
      }
      if (ok && !aborted(abort_flag)) {
        // every stage released: no commit from the even CTA is still on its
        // way to this CTA's barriers
        for (int i = 0; i < PSTAGES; ++i) {
          if (!mbar_wait_bounded(&empty[stage], ph ^ 1)) {
            report_status(status, DEV_TIMEOUT_EMPTY);
            *abort_flag = 1;
            break;
          }
          if (++stage == PSTAGES) {
            stage = 0;
            ph ^= 1;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------ MMA issuer (even CTA) ------------------------------
    if (lane == 0 && leader) {
      const uint32_t idv = tc::idesc(tc::kind_fmt(KIND), 2 * BM, BN);
      int stage = 0;
      uint32_t ph = 0;
      int buf = 0;
      uint32_t acc_ph[2] = {0, 0};
      auto issue = [&](const Params& P, const CUtensorMap*, const CUtensorMap*, int64_t t) -> bool {
        int g0, g1;
        groups_of(P, t, g0, g1);
        for (int g = g0; g < g1; ++g) {
          int load = 0;
          bool open = false;
          uint32_t d_tmem = 0;
          for (int pp = P.group_begin[g]; pp < P.group_begin[g + 1]; ++pp) {
            const int w = P.pair_w[pp];
            if (open && !P.merge_pairs) {
              tc::commit2_mc(&tfull[buf], (uint16_t)0x3);
              acc_ph[buf] ^= 1;
              buf ^= 1;
              open = false;
            }
            for (int st = 0; st < P.kblocks;) {
              if (open && load + w > P.chunk_cap) {
                tc::commit2_mc(&tfull[buf], (uint16_t)0x3);
                acc_ph[buf] ^= 1;
                buf ^= 1;
                open = false;
              }
              bool fresh = false;
              if (!open) {
                if (!mbar_wait_bounded(&tempty[buf], acc_ph[buf] ^ 1)) {
                  report_status(status, DEV_TIMEOUT_TMEM);
                  *abort_flag = 1;
                  return false;
                }
                tc::fence_after();
                d_tmem = tmem_base + (uint32_t)(buf * BN);
                load = 0;
                open = fresh = true;
              }
              // the k-blocks of this pair that still fit in the open chunk
              const int s0 = st, s1 = min(P.kblocks, st + (P.chunk_cap - load) / w);
              for (; st < s1; ++st) {
                if (!mbar_wait_bounded(&full[stage], ph)) {
                  report_status(status, DEV_TIMEOUT_FULL);
                  *abort_flag = 1;
                  return false;
                }
                tc::fence_after();
                const uint32_t a_addr = smem_u32(smem + stage * P_STAGE_BYTES);
                const uint32_t b_addr = a_addr + A_TILE;
#pragma unroll
                for (int kk = 0; kk < KSTEPS; ++kk)
                  tc::mma2<KIND>(d_tmem, tc::sdesc_k128(a_addr + kk * 32), tc::sdesc_k128(b_addr + kk * 32), idv,
                                (fresh && st == s0 && kk == 0) ? 0u : 1u);
                tc::commit2_mc(&empty[stage], (uint16_t)0x3);
                if (++stage == PSTAGES) {
                  stage = 0;
                  ph ^= 1;
                }
              }
              load += (s1 - s0) * w;
            }
          }
          if (open) {
            tc::commit2_mc(&tfull[buf], (uint16_t)0x3);
            acc_ph[buf] ^= 1;
            buf ^= 1;
          }
        }
        return true;
      };
      bool ok = true;
      for (int64_t r = 0; r * unit_step < units && ok && !aborted(abort_flag); ++r) {
        const int64_t u = unit_at(r);
        if (u >= units) continue;
        ok = with_unit(u, issue);
      }
      if (aborted(abort_flag)) {
        tc::commit2_mc(drain, (uint16_t)0x1);
        mbar_wait_bounded(drain, 0);
      }
    }
  } else {
    // ------------------------------ epilogue (both CTAs) ------------------------------
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    const int r_local = q * 32 + lane;
    const uint32_t tempty_leader[2] = {mapa_shared(&tempty[0], 0), mapa_shared(&tempty[1], 0)};
    int buf = 0;
    uint32_t acc_ph[2] = {0, 0};
    auto drain_unit = [&](const Params& P, const CUtensorMap*, const CUtensorMap*, int64_t t) -> bool {
      int tm, tn, g0, g1;
      coords(P, t, tm, tn);
      groups_of(P, t, g0, g1);
      const int64_t row = (int64_t)tm * BM + r_local;
      const int64_t col0 = (int64_t)tn * BN + h * EPI_COLS;
      if (EPI == EPI_F32) prefetch_c_rows<EPI_COLS>(P, (int64_t)tm * BM + q * 32, col0, lane);
      EpiAcc<EPI> S[EPI_COLS];
#pragma unroll
      for (int j = 0; j < EPI_COLS; ++j) S[j] = EpiAcc<EPI>(0);
      for (int g = g0; g < g1; ++g) {
        for (int c = 0; c < P.group_chunks[g]; ++c) {
          if (!mbar_wait_bounded(&tfull[buf], acc_ph[buf])) {
            report_status(status, DEV_TIMEOUT_MMA);
            *abort_flag = 1;
            return false;
          }
          tc::fence_after();
          const uint32_t taddr = tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN + h * EPI_COLS);
          drain_chunk<EPI, EPI_COLS>(taddr, S);
          tc::fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster_relaxed(tempty_leader[buf]);
          acc_ph[buf] ^= 1;
          buf ^= 1;
        }
        if (EPI == EPI_OZAKI) {
          if (row < P.m) {
            // tile-blocked plane: this CTA's 128 x 256 tile is one contiguous
            // block, column after column of 128 rows (see the host's plane layout)
            int* srow = P.sbuf + (size_t)g * P.plane + (size_t)tn * ((size_t)P.tiles_m * BM * BN) +
                        (size_t)tm * (BM * BN) + (size_t)(h * EPI_COLS) * BM + r_local;
#pragma unroll
            for (int j = 0; j < EPI_COLS; ++j) {
              const int64_t col = col0 + j;
              if (col < P.n) srow[j * BM] = S[j];
            }
          }
#pragma unroll
          for (int j = 0; j < EPI_COLS; ++j) S[j] = EpiAcc<EPI>(0);
        }
      }
      if constexpr (EPI == EPI_BOUND) bound_tile<EPI_COLS>(P, row, col0, S);
      if (EPI == EPI_F32 && row < P.m) {
        // C is read 8 columns at a time, every load of a group issued before
        // the first use (one memory round trip per group, not per element)
        float* crow = P.c32 + row * P.rsc;
#pragma unroll
        for (int j0 = 0; j0 < EPI_COLS; j0 += 8) {
          float c0[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t col = col0 + j0 + j;
            c0[j] = (P.beta_f != 0.0f && col < P.n) ? crow[col * P.csc] : 0.0f;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int64_t col = col0 + j0 + j;
            if (col < P.n) {
              const float v = (float)S[j0 + j] * P.alpha_f;
              crow[col * P.csc] = (P.beta_f == 0.0f) ? v : fmaf(P.beta_f, c0[j], v);
            }
          }
        }
      }
      return true;
    };
    bool ok = true;
    for (int64_t r = 0; r * unit_step < units && ok && !aborted(abort_flag); ++r) {
      const int64_t u = unit_at(r);
      if (u >= units) continue;
      ok = with_unit(u, drain_unit);
    }
  }

  __syncwarp();
  tc::fence_before();
  __syncthreads();
  cluster_sync();  // both CTAs are done with each other's barriers and TMEM
  if (warp == 1) {
    tc::fence_after();
    tc::tmem_dealloc2(tmem_base, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// Chunk counts of every group (Params::group_chunks) under the chunk rule
// the MMA issuer applies step by step: a chunk takes a pair's k-blocks while
// their weights fit in chunk_cap, continues into the next pair only with
// merge_pairs, and a new chunk holds floor(chunk_cap / w) k-blocks of a pair
// of weight w. Returns false if a weight exceeds the capacity.
inline bool plan_chunks(Params& p) {
  const int cap = p.chunk_cap;
  for (int g = 0; g < p.ngroups; ++g) {
    int n = 0, load = 0;
    bool open = false;
    for (int pp = p.group_begin[g]; pp < p.group_begin[g + 1]; ++pp) {
      const int w = p.pair_w[pp];
      if (w < 1 || w > cap) return false;
      int rem = p.kblocks;
      if (open && p.merge_pairs) {
        const int take = std::min(rem, (cap - load) / w);
        rem -= take;
        load += take * w;
      } else {
        open = false;
      }
      if (rem > 0) {
        const int per = cap / w;
        const int fresh = (rem + per - 1) / per;
        n += fresh;
        load = (rem - (fresh - 1) * per) * w;
        open = true;
      }
    }
    p.group_chunks[g] = n;
  }
  return true;
}

template <int KIND, int EPI>
inline cudaError_t set_slice_attrs() {
  cudaError_t e = cudaFuncSetAttribute(slice_gemm_kernel<KIND, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       SMEM_BYTES);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(slice_gemm_pair_kernel<KIND, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             P_SMEM_BYTES);
  if (e == cudaSuccess && EPI == EPI_OZAKI)
    e = cudaFuncSetAttribute(slice_gemm_pair_kernel<KIND, EPI, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             P_SMEM_BYTES);
  return e;
}

// Kernel variants: 0 = one CTA per tile, 2 = CTA pairs with cta_group::2 MMA
// (1 is not used: it was a cluster kernel sharing B tiles by multicast loads).
enum { SLICE_SINGLE = 0, SLICE_PAIR = 2 };

inline cudaLaunchConfig_t cluster2_config(int smem, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = (size_t)smem;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// The variant to use on the current device and how many CTA pairs fit at
// once; queried once per device. MOMMS_SLICE_VARIANT=0 restricts the choice to
// the single-CTA kernel (default and MOMMS_SLICE_VARIANT=2: the pair kernel
// wherever the device can co-schedule pairs).
template <int KIND, int EPI>
inline int slice_variant(int* clusters) {
  static std::atomic<int> cache_v[64], cache_n[64];
  static std::atomic<bool> init[64];
  int dev = 0;
  *clusters = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SLICE_SINGLE;
  if (!init[dev].load()) {
    const char* env = getenv("MOMMS_SLICE_VARIANT");
    const bool want_pair = !(env && env[0] == '0');
    int v = SLICE_SINGLE, n = 0;
    if (want_pair) {
      cudaLaunchAttribute attr[1];
      cudaLaunchConfig_t cfg = cluster2_config(P_SMEM_BYTES, attr);
      int c = 0;
      if (cudaOccupancyMaxActiveClusters(&c, (const void*)slice_gemm_pair_kernel<KIND, EPI>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        c = 0;
      }
      if (c > 0) {
        v = SLICE_PAIR;
        n = c;
      }
    }
    cache_v[dev].store(v);
    cache_n[dev].store(n);
    init[dev].store(true);
  }
  *clusters = cache_n[dev].load();
  return cache_v[dev].load();
}

// Launches the slice kernel. The pair kernel needs at least two m-tiles (its
// units are vertical tile pairs) and takes tmB_half, whose box is BN/2 rows
// (each CTA of a pair stages its half of the B tile); the single-CTA kernel
// takes tmB_full. *variant receives the one run.
template <int KIND, int EPI>
inline cudaError_t launch_slice(const CUtensorMap& tmA, const CUtensorMap& tmB_full, const CUtensorMap& tmB_half,
                                const Params& p, int sm_count, cudaStream_t s, int* variant) {
  int clusters = 0;
  const int v = p.tiles_m >= 2 ? slice_variant<KIND, EPI>(&clusters) : SLICE_SINGLE;
  *variant = v;
  const int64_t tile_units = v == SLICE_PAIR ? (int64_t)((p.tiles_m + 1) / 2) * p.tiles_n
                                             : (int64_t)p.tiles_m * p.tiles_n;
  const int64_t slots = v == SLICE_PAIR ? clusters : sm_count;
  Params q = p;
  if (!plan_chunks(q)) return cudaErrorInvalidValue;
  q.gchunk = p.ngroups;
  // Few tiles: a tile's accumulation groups (each writes its own int32 plane)
  // can run as separate work units. Pick the split whose schedule of units
  // (group-major, handed out in the kernel's snake order; cost = k-blocks of
  // the unit's pairs plus 8 for its pipeline fill) finishes first.
  if (EPI == EPI_OZAKI && tile_units < 4 * slots && p.ngroups > 1) {
    double best = -1.0;
    std::vector<double> load((size_t)slots);
    for (int gc = p.ngroups; gc >= 1; gc = gc == 1 ? 0 : (gc + 1) / 2) {
      std::fill(load.begin(), load.end(), 0.0);
      const int chunks = (p.ngroups + gc - 1) / gc;
      int64_t u = 0;
      for (int c = 0; c < chunks; ++c) {
        const int g0 = c * gc, g1 = std::min(p.ngroups, g0 + gc);
        const double cost = 8.0 + (double)(p.group_begin[g1] - p.group_begin[g0]) * (double)p.kblocks;
        for (int64_t tu = 0; tu < tile_units; ++tu, ++u) {
          const int64_t r = u / slots, i = u % slots;
          load[(size_t)((r & 1) ? slots - 1 - i : i)] += cost;  // the kernel's snake order
        }
      }
      const double makespan = *std::max_element(load.begin(), load.end());
      if (best < 0.0 || makespan < best * 0.97) {  // a finer split must gain 3 %
        best = makespan;
        q.gchunk = gc;
      }
    }
  }
  const int64_t units = tile_units * ((p.ngroups + q.gchunk - 1) / q.gchunk);
  if (v == SLICE_PAIR) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = cluster2_config(P_SMEM_BYTES, attr);
    cfg.gridDim = dim3((unsigned)(2 * std::min<int64_t>(units, clusters)));
    cfg.stream = s;
    return cudaLaunchKernelEx(&cfg, slice_gemm_pair_kernel<KIND, EPI>, tmA, tmB_half, q, GroupTable{});
  }
  const int grid = (int)std::min<int64_t>(units, sm_count);
  slice_gemm_kernel<KIND, EPI><<<grid, THREADS, SMEM_BYTES, s>>>(tmA, tmB_full, q);
  return cudaGetLastError();
}

}  // namespace sp
}  // namespace momms
