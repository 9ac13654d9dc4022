// Operand -> K-major precision planes, the pre-pass of the tcgen05 paths.
//
// An operand is viewed as R x K (A: R = m; B transposed: R = n), element
// (r, p) at x[r*sr + p*sp]. Each element is split by `Op` into NP values that
// are written to planes[t][r][p] (p contiguous, row stride ldp, plane stride
// plane_elems). A 32 x 32 shared-memory tile makes both the read (along
// whichever index is contiguous in the source) and the write (along p)
// coalesced.
#pragma once
#include "common.cuh"

namespace momms {
namespace planes {

constexpr int TILE = 32, ROWS_PER_PASS = 8;

template <typename Tin, typename Op>
__global__ void __launch_bounds__(TILE* ROWS_PER_PASS)
    to_planes_kernel(const Tin* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K, bool r_contig,
                     typename Op::Tout* __restrict__ planes, int64_t ldp, int64_t plane_elems, Op op) {
  __shared__ Tin tile[TILE][TILE + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r0 = (int64_t)blockIdx.y * TILE, p0 = (int64_t)blockIdx.x * TILE;
#pragma unroll
  for (int i = 0; i < TILE / ROWS_PER_PASS; ++i) {
    const int a = tx, b = ty + i * ROWS_PER_PASS;
    // tx walks the source's contiguous index
    const int rl = r_contig ? a : b, pl = r_contig ? b : a;
    const int64_t r = r0 + rl, pp = p0 + pl;
    tile[rl][pl] = (r < R && pp < K) ? x[r * sr + pp * sp] : Tin(0);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < TILE / ROWS_PER_PASS; ++i) {
    const int rl = ty + i * ROWS_PER_PASS, pl = tx;
    const int64_t r = r0 + rl, pp = p0 + pl;
    if (r < R && pp < K) op(tile[rl][pl], r, planes + r * ldp + pp, plane_elems);
  }
}

template <typename Tin, typename Op>
void launch_to_planes(const Tin* x, int64_t sr, int64_t sp, int64_t R, int64_t K, typename Op::Tout* planes,
                      int64_t ldp, int64_t plane_elems, Op op, cudaStream_t s) {
  const bool r_contig = (sr == 1 && sp != 1);
  dim3 block(TILE, ROWS_PER_PASS);
  dim3 grid((unsigned)ceil_div_dev(K, TILE), (unsigned)ceil_div_dev(R, TILE));
  to_planes_kernel<Tin, Op><<<grid, block, 0, s>>>(x, sr, sp, R, K, r_contig, planes, ldp, plane_elems, op);
}

}  // namespace planes
}  // namespace momms
