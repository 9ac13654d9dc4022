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

template <typename Tin, typename Op>
__global__ void __launch_bounds__(THREADS, 4)
    to_planes_kernel(const Tin* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K, bool r_contig,
                     typename Op::Tout* __restrict__ planes, int64_t ldp, int64_t plane_elems, Op op) {
  __shared__ Tin tile[TILE_R][TILE_P + 1];
  const int tid = threadIdx.x;
  const int64_t p0 = (int64_t)blockIdx.x * TILE_P;
  // row tiles beyond the grid's y limit are taken in further passes
  for (int64_t r0 = (int64_t)blockIdx.y * TILE_R; r0 < R; r0 += (int64_t)gridDim.y * TILE_R) {
    __syncthreads();  // the previous pass's readers are done with the tile
#pragma unroll
    for (int i = 0; i < TILE_R * TILE_P / THREADS; ++i) {
      const int lin = tid + THREADS * i;
      // consecutive threads walk the source's contiguous index
      const int rl = r_contig ? (lin % TILE_R) : (lin / TILE_P);
      const int pl = r_contig ? (lin / TILE_R) : (lin % TILE_P);
      const int64_t r = r0 + rl, pp = p0 + pl;
      tile[rl][pl] = (r < R && pp < K) ? x[r * sr + pp * sp] : Tin(0);
    }
    __syncthreads();
#pragma unroll 1
    for (int i = 0; i < TILE_R * (TILE_P / 2) / THREADS; ++i) {
      const int item = tid + THREADS * i;
      const int pr = item % (TILE_P / 2), rl = item / (TILE_P / 2);
      const int64_t r = r0 + rl, pp = p0 + 2 * pr;
      if (r < R && pp < K) op.pair(tile[rl][2 * pr], tile[rl][2 * pr + 1], r, planes + r * ldp + pp, plane_elems);
    }
  }
}

template <typename Tin, typename Op>
void launch_to_planes(const Tin* x, int64_t sr, int64_t sp, int64_t R, int64_t K, typename Op::Tout* planes,
                      int64_t ldp, int64_t plane_elems, Op op, cudaStream_t s) {
  const bool r_contig = (sr == 1 && sp != 1);
  dim3 grid((unsigned)ceil_div_dev(K, TILE_P), (unsigned)std::min<int64_t>(ceil_div_dev(R, TILE_R), 65535));
  to_planes_kernel<Tin, Op><<<grid, THREADS, 0, s>>>(x, sr, sp, R, K, r_contig, planes, ldp, plane_elems, op);
}

}  // namespace planes
}  // namespace momms
