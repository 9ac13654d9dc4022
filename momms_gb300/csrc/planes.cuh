// Operand -> K-major precision planes, the pre-pass of the tcgen05 paths.
//
// An operand is viewed as R x K (A: R = m; B transposed: R = n), element
// (r, p) at x[r*sr + p*sp]. Each element is split by `Op` into values written
// to planes[t][r][p] (p contiguous, row stride ldp, plane stride
// plane_elems).
//
// Work is cut into runs: RUN consecutive elements of one row, RUN * sizeof
// of the plane type = 16 bytes, so that a run's values of one plane leave in
// one vector store. The warp layout follows the source's contiguous index:
//   * rows contiguous (a column-major A): a warp takes 4 consecutive rows x
//     8 consecutive runs (lane = 4 * run + row), so each of a thread's RUN
//     loads reads eight 32-byte pieces (4 rows of 8 columns) and each plane
//     store writes 128 contiguous bytes (8 runs) of each of 4 rows: whole
//     lines. (With a warp on 32 rows of one run, every store was 32 separate
//     16-byte pieces, one L2 write request each, and the digit pass was
//     store-throttled. The read-only and single-plane passes use 8 rows x 4
//     runs, see kRowsContigLg.)
//   * otherwise (p contiguous, or general strides): the lanes take 32
//     consecutive runs of one row, read with 16-byte vector loads where the
//     row is aligned, and each plane store is one contiguous 512-byte warp
//     access. Rows shorter than 32 runs share a warp: 2^lg lanes per row,
//     2^lg the smallest power of two covering the row's runs.
// Nothing goes through shared memory and nothing waits at a barrier. A
// thread converts PITER runs of its row, each `runs` runs after the last
// (the runs of the warp's other lanes on that row lie in between).
// (Loading the next run while converting the current one took more
// registers than it hid latency: 0.277 -> 0.284 ms for the digits of A,
// 0.14 -> 0.17 ms for the magnitudes, at 8192^2.)
// Requires ldp, plane_elems and the plane base aligned to RUN elements
// (16 bytes); the last run of a row may extend past K up to
// round_up(K, RUN) <= ldp, and those padding columns receive the split of zero.
#pragma once
#include "common.cuh"

namespace momms {
void refuse_launch(cudaError_t e);
namespace planes {

constexpr int THREADS = 256, PITER = 4;

// A thread's place in a block's chunk of the view: row rl of the chunk's
// rows, run ru of the runs taken across the chunk per iteration. A warp
// holds 32 >> lg rows of 2^lg runs each; rows contiguous: consecutive lanes
// take consecutive rows (lane = run * rows_per_warp + row), otherwise
// consecutive runs of a row. Host-callable, so that the index arithmetic is
// checked on the CPU.
struct RunPlace {
  int rows, runs, rl, ru;
};
template <bool R_CONTIG>
__host__ __device__ __forceinline__ RunPlace run_place(int tid, int lg) {
  const int lane = tid & 31, warp = tid >> 5;
  RunPlace c;
  if (R_CONTIG) {
    const int rpw = 32 >> lg;
    c.rows = (THREADS / 32) * rpw, c.runs = 1 << lg, c.rl = warp * rpw + (lane & (rpw - 1)), c.ru = lane >> (5 - lg);
  } else {
    c.rows = (THREADS / 32) << (5 - lg), c.runs = 1 << lg;
    c.rl = (warp << (5 - lg)) + (lane >> lg), c.ru = lane & (c.runs - 1);
  }
  return c;
}
// First column of the thread's run `it` in block column bx (runs of `run`
// elements; a block covers runs * run * PITER columns).
__host__ __device__ __forceinline__ int64_t run_col(int64_t bx, const RunPlace& c, int it, int run) {
  return (bx * c.runs * PITER + c.ru + (int64_t)c.runs * it) * run;
}
template <bool R_CONTIG>
struct Chunk : RunPlace {
  __device__ __forceinline__ explicit Chunk(int lg) : RunPlace(run_place<R_CONTIG>((int)threadIdx.x, lg)) {}
};

// Lanes per row (log2) for rows of K elements in runs of RUN: rows not
// contiguous, the smallest power of two covering the row's runs (at most
// 32); rows contiguous, `rows_contig_lg` capped the same way.
inline int run_lanes_log2(int64_t K, int run, bool r_contig, int rows_contig_lg) {
  const int64_t runs = (K + run - 1) / run;
  int lg = 0;
  while (lg < 5 && ((int64_t)1 << lg) < runs) ++lg;
  return r_contig ? std::min(lg, rows_contig_lg) : lg;
}
// Rows-contiguous lanes per row (log2) of the prep kernels. Digits of an
// 8192^2 A (7 planes per run): 8 runs x 4 rows 0.243 ms, 4 runs x 8 rows
// 0.277 ms, 2 x 16 0.352 ms, 1 x 32 1.02 ms (16-byte row pieces, one L2 write
// request each). The magnitudes (one plane) and row maxima read alike at
// every shape tried and keep 4 runs x 8 rows.
constexpr int kRowsContigLg = 2, kRowsContigLgPlanes = 3;

// Loads the run of row xr starting at p (p a multiple of RUN): RUN elements,
// zeros past K. `vec`: p contiguous and the row 16-byte aligned, so the run
// is read with 16-byte vector loads.
template <bool R_CONTIG, int RUN, typename Tin>
__device__ __forceinline__ void load_run(const Tin* __restrict__ xr, int64_t sp, int64_t p, int64_t K, bool vec,
                                         Tin (&v)[RUN]) {
  static_assert((RUN * sizeof(Tin)) % 16 == 0, "a run is whole 16-byte vectors");
  if (p + RUN <= K) {
    if (!R_CONTIG && vec) {
      const uint4* q = reinterpret_cast<const uint4*>(xr + p);
      uint4 t[RUN * sizeof(Tin) / 16];
#pragma unroll
      for (int i = 0; i < RUN * (int)sizeof(Tin) / 16; ++i) t[i] = __ldg(q + i);
      memcpy(v, t, sizeof(v));
    } else {
      const Tin* q = xr + p * sp;
#pragma unroll
      for (int i = 0; i < RUN; ++i) v[i] = __ldg(q + i * sp);
    }
  } else {
#pragma unroll
    for (int i = 0; i < RUN; ++i) v[i] = (p + i < K) ? __ldg(xr + (p + i) * sp) : Tin(0);
  }
}

// Op: PLANES, Tout, Word (one pair's value in one plane: two Tout), Ctx
// row(r) (per-row state) and pack(v0, v1, ctx, Word (&w)[PLANES]).
template <bool R_CONTIG, typename Tin, typename Op>
__global__ void __launch_bounds__(THREADS)
    to_planes_kernel(const Tin* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K, bool vec, int lg,
                     typename Op::Tout* __restrict__ planes, int64_t ldp, int64_t plane_elems, Op op) {
  using Tout = typename Op::Tout;
  using Word = typename Op::Word;
  constexpr int RUN = 16 / sizeof(Tout), NP = Op::PLANES;
  static_assert(sizeof(Word) == 2 * sizeof(Tout), "a word is one pair's value");
  const Chunk<R_CONTIG> c(lg);
  // row chunks beyond the grid's y limit are taken in further passes
  for (int64_t r = (int64_t)blockIdx.y * c.rows + c.rl; r < R; r += (int64_t)gridDim.y * c.rows) {
    const auto ctx = op.row(r);
    const Tin* xr = x + r * sr;
    Tout* outr = planes + r * ldp;
#pragma unroll 1
    for (int it = 0; it < PITER; ++it) {
      const int64_t p = run_col(blockIdx.x, c, it, RUN);
      if (p >= K) break;
      Tin v[RUN];
      load_run<R_CONTIG, RUN>(xr, sp, p, K, vec, v);
      Word w[NP][RUN / 2];
#pragma unroll
      for (int q = 0; q < RUN / 2; ++q) {
        Word wq[NP];
        op.pack(v[2 * q], v[2 * q + 1], ctx, wq);
#pragma unroll
        for (int t = 0; t < NP; ++t) w[t][q] = wq[t];
      }
#pragma unroll
      for (int t = 0; t < NP; ++t) {
        uint4 u;
        memcpy(&u, w[t], sizeof(u));
        *reinterpret_cast<uint4*>(outr + t * plane_elems + p) = u;
      }
    }
  }
}

// Grid of a run kernel over an R x K view, lg from run_lanes_log2: a block
// holds 256 >> lg rows of 2^lg runs in either layout (the layouts differ in
// which lanes take which place, run_place). Rows past 65535 blocks are taken
// by the kernels' row loops.
template <bool R_CONTIG, int RUN>
inline dim3 run_grid(int64_t R, int64_t K, int lg) {
  const int64_t rows = (int64_t)(THREADS / 32) << (5 - lg);
  const int64_t runs = (int64_t)1 << lg;
  return dim3((unsigned)ceil_div_dev(K, runs * RUN * PITER), (unsigned)std::min<int64_t>(ceil_div_dev(R, rows), 65535));
}

// True when row r of the view starts 16-byte aligned for every r and p is
// contiguous, so that runs may be read as vectors.
template <typename Tin>
inline bool rows_vector_aligned(const Tin* x, int64_t sr, int64_t sp) {
  return sp == 1 && (reinterpret_cast<uintptr_t>(x) & 15) == 0 && ((sr * (int64_t)sizeof(Tin)) & 15) == 0;
}

template <typename Tin, typename Op>
void launch_to_planes(const Tin* x, int64_t sr, int64_t sp, int64_t R, int64_t K, typename Op::Tout* planes,
                      int64_t ldp, int64_t plane_elems, Op op, cudaStream_t s) {
  constexpr int RUN = 16 / sizeof(typename Op::Tout);
  if (ldp % RUN || plane_elems % RUN || (reinterpret_cast<uintptr_t>(planes) & 15)) {
    refuse_launch(cudaErrorMisalignedAddress);  // the vector stores need 16-byte aligned runs
    return;
  }
  const bool r_contig = (sr == 1 && sp != 1);
  const bool vec = rows_vector_aligned(x, sr, sp);
  const int lg = run_lanes_log2(K, RUN, r_contig, kRowsContigLgPlanes);
  if (r_contig)
    to_planes_kernel<true, Tin, Op>
        <<<run_grid<true, RUN>(R, K, lg), THREADS, 0, s>>>(x, sr, sp, R, K, vec, lg, planes, ldp, plane_elems, op);
  else
    to_planes_kernel<false, Tin, Op>
        <<<run_grid<false, RUN>(R, K, lg), THREADS, 0, s>>>(x, sr, sp, R, K, vec, lg, planes, ldp, plane_elems, op);
}

}  // namespace planes
}  // namespace momms
