// Operand -> K-major precision planes, the pre-pass of the tcgen05 paths.
//
// An operand is viewed as R x K (A: R = m; B transposed: R = n), element
// (r, p) at x[r*sr + p*sp]. Each element is split by `Op` into values written
// to planes[t][r][p] (p contiguous, row stride ldp, plane stride
// plane_elems). A block stages a 32 x 64 tile in shared memory so that the
// read (along whichever index is contiguous in the source) and the write
// (along p) are both coalesced; each thread then splits two neighbouring
// elements of a row and stores each plane's pair as one vector (a warp writes
// 128 contiguous bytes of fp16 per plane). Requires ldp and plane_elems even
// and `planes` 8-byte aligned; the pair at the end of an odd K covers a
// padding column (p = K <= ldp - 1), which receives the split of zero.
#pragma once
#include "common.cuh"

namespace momms {
namespace planes {

constexpr int TILE_R = 32, TILE_P = 64, THREADS = 256;

// Stages rows r0..r0+31, columns p0..p0+63 of the view into tile (zeros
// outside it). Every thread's element of pass i lies a fixed distance from
// its element of pass 0 (8 columns on when rows are contiguous, 4 rows on
// otherwise), so a pass costs one pointer step; interior tiles skip the
// bounds checks.
template <bool R_CONTIG, typename Tin>
__device__ __forceinline__ void stage_tile(const Tin* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K,
                                           int64_t r0, int64_t p0, Tin (&tile)[TILE_R][TILE_P + 1]) {
  const int tid = threadIdx.x;
  // pass i: rows-contiguous (rl, pl) = (tid % 32, tid / 32 + 8 i), else (tid / 64 + 4 i, tid % 64)
  const int rl0 = R_CONTIG ? (tid % TILE_R) : (tid / TILE_P);
  const int pl0 = R_CONTIG ? (tid / TILE_R) : (tid % TILE_P);
  constexpr int DR = R_CONTIG ? 0 : THREADS / TILE_P, DP = R_CONTIG ? THREADS / TILE_R : 0;
  const Tin* q = x + (r0 + rl0) * sr + (p0 + pl0) * sp;
  const int64_t step = R_CONTIG ? (int64_t)DP * sp : (int64_t)DR * sr;
  constexpr int PASSES = TILE_R * TILE_P / THREADS;
  if (r0 + TILE_R <= R && p0 + TILE_P <= K) {
    Tin v[PASSES];
#pragma unroll
    for (int i = 0; i < PASSES; ++i) v[i] = q[i * step];
#pragma unroll
    for (int i = 0; i < PASSES; ++i) tile[rl0 + DR * i][pl0 + DP * i] = v[i];
  } else {
#pragma unroll
    for (int i = 0; i < PASSES; ++i) {
      const int rl = rl0 + DR * i, pl = pl0 + DP * i;
      tile[rl][pl] = (r0 + rl < R && p0 + pl < K) ? q[i * step] : Tin(0);
    }
  }
}

template <bool R_CONTIG, typename Tin, typename Op>
__global__ void __launch_bounds__(THREADS, 4)
    to_planes_kernel(const Tin* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K,
                     typename Op::Tout* __restrict__ planes, int64_t ldp, int64_t plane_elems, Op op) {
  __shared__ Tin tile[TILE_R][TILE_P + 1];
  const int tid = threadIdx.x;
  const int64_t p0 = (int64_t)blockIdx.x * TILE_P;
  // a thread splits the pair at column 2 (tid % 32) of rows tid / 32 + 8 i
  const int pr = tid % (TILE_P / 2), rl0 = tid / (TILE_P / 2);
  const int64_t pp = p0 + 2 * pr;
  // row tiles beyond the grid's y limit are taken in further passes
  for (int64_t r0 = (int64_t)blockIdx.y * TILE_R; r0 < R; r0 += (int64_t)gridDim.y * TILE_R) {
    __syncthreads();  // the previous pass's readers are done with the tile
    stage_tile<R_CONTIG>(x, sr, sp, R, K, r0, p0, tile);
    __syncthreads();
    if (pp >= K) continue;
    typename Op::Tout* out = planes + (r0 + rl0) * ldp + pp;
#pragma unroll 1
    for (int i = 0; i < TILE_R * (TILE_P / 2) / THREADS; ++i) {
      const int rl = rl0 + (THREADS / (TILE_P / 2)) * i;
      if (r0 + rl >= R) break;
      op.pair(tile[rl][2 * pr], tile[rl][2 * pr + 1], r0 + rl, out, plane_elems);
      out += (int64_t)(THREADS / (TILE_P / 2)) * ldp;
    }
  }
}

template <typename Tin, typename Op>
void launch_to_planes(const Tin* x, int64_t sr, int64_t sp, int64_t R, int64_t K, typename Op::Tout* planes,
                      int64_t ldp, int64_t plane_elems, Op op, cudaStream_t s) {
  const bool r_contig = (sr == 1 && sp != 1);
  dim3 grid((unsigned)ceil_div_dev(K, TILE_P), (unsigned)std::min<int64_t>(ceil_div_dev(R, TILE_R), 65535));
  if (r_contig) to_planes_kernel<true, Tin, Op><<<grid, THREADS, 0, s>>>(x, sr, sp, R, K, planes, ldp, plane_elems, op);
  else to_planes_kernel<false, Tin, Op><<<grid, THREADS, 0, s>>>(x, sr, sp, R, K, planes, ldp, plane_elems, op);
}

}  // namespace planes
}  // namespace momms
