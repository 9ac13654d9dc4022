// Plain f32 GEMM on the FP32 pipes: register-blocked FFMA.
//
// The GPU form of the reference's f32 path (the bli_sgemm_haswell_asm_6x16
// register block, ukernels/bli_gemm_haswell_asm_d6x8.c:77-640, under the same
// Goto loops): a persistent 128 x 128 CTA tile, 256 threads each owning an
// 8 x 8 register block, k streamed in blocks of 16 through double-buffered
// shared memory. Global loads are 128-bit and coalesced along whichever index
// of the operand is contiguous; k-contiguous operands are transposed on their
// way into shared memory so that every inner-loop read is a conflict-free
// 128-bit load. Each output element is a sequential fma chain over k (the
// microkernel's order, d6x8.c:725-885), then acc*alpha, then
// fma(beta, c, acc).
#include "ffma_core.cuh"
#include "internal.h"

namespace momms {
namespace ffma {

struct Params {
  Operands o;
  Epi e;
  TileSched sched;
  float* partials;
  unsigned* counters;
};

// SPLIT: the launch splits k (p.sched.splits > 1); without it the unit loop
// carries no split bookkeeping, which keeps the main loop within 128
// registers (2 CTAs of 256 threads, or 8 of 64, per SM) without spilling.
// TM: the tile edge (128 or 64).
template <int TM, bool A_XC, bool B_XC, typename Off, bool SPLIT>
__global__ void __launch_bounds__(Tile<TM>::THREADS, Tile<TM>::CTAS_PER_SM)
    sgemm_kernel(const __grid_constant__ Params p) {
  extern __shared__ float4 ffma_smem[];
  __shared__ int s_last;
  const Operands& o = p.o;
  const int64_t units = p.sched.units();
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    int tm, tn, sp;
    p.sched.decode(u, tm, tn, sp);
    const int64_t kblocks = ceil_div_dev(o.k, BK);
    const int64_t kb0 = SPLIT ? sp * (p.sched.k_per_split / BK) : 0;
    const int64_t kb1 = SPLIT ? min(kblocks, kb0 + p.sched.k_per_split / BK) : kblocks;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    prefetch_c_tile<TM>(p.e, tm, tn);
    ffma_unit_t<TM, A_XC, B_XC, Off>(o, tm, tn, kb0, kb1, acc, reinterpret_cast<float*>(ffma_smem));
    if (SPLIT) {
      const int64_t tile = u / p.sched.splits;
      ffma_finish<TM>(p.e, acc, tm, tn, p.sched.splits, sp, p.partials + (size_t)tile * p.sched.splits * TM * TM,
                      p.counters + tile, &s_last);
    } else {
      ffma_finish<TM>(p.e, acc, tm, tn, 1, 0, nullptr, nullptr, &s_last);
    }
  }
}

typedef void (*Kern)(const Params);
// The instantiations of one tile size, by [A layout][B layout][offset width][split].
template <int TM>
const Kern (&kernel_table())[2][2][2][2] {
  static const Kern t[2][2][2][2] = {
      {{{sgemm_kernel<TM, false, false, uint32_t, false>, sgemm_kernel<TM, false, false, uint32_t, true>},
        {sgemm_kernel<TM, false, false, uint64_t, false>, sgemm_kernel<TM, false, false, uint64_t, true>}},
       {{sgemm_kernel<TM, false, true, uint32_t, false>, sgemm_kernel<TM, false, true, uint32_t, true>},
        {sgemm_kernel<TM, false, true, uint64_t, false>, sgemm_kernel<TM, false, true, uint64_t, true>}}},
      {{{sgemm_kernel<TM, true, false, uint32_t, false>, sgemm_kernel<TM, true, false, uint32_t, true>},
        {sgemm_kernel<TM, true, false, uint64_t, false>, sgemm_kernel<TM, true, false, uint64_t, true>}},
       {{sgemm_kernel<TM, true, true, uint32_t, false>, sgemm_kernel<TM, true, true, uint32_t, true>},
        {sgemm_kernel<TM, true, true, uint64_t, false>, sgemm_kernel<TM, true, true, uint64_t, true>}}}};
  return t;
}

}  // namespace ffma

namespace {
// The launcher proper; scratch[0..2] (repacked A, B, split-k workspace) are
// returned to the pool by the caller, on every path.
int sgemm_ffma_impl(const DevGemm& g0, cudaStream_t s, void* (&scratch)[3]) {
  using namespace ffma;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  DevGemm g = g0;
  cudaError_t ce;
  if ((ce = wait_operands(g, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
  // A must have unit stride along m or k; B along k or n. Anything else is
  // first copied into a column-major scratch matrix.
  auto unit = [](const DevMat& v, int64_t, int64_t) { return v.rs == 1 || v.cs == 1; };
  if (!unit(g.a, g.m, g.k)) {
    int64_t ld = round_up(g.m, 4);
    if ((ce = scratch_alloc(&scratch[0], (size_t)ld * g.k * 4, s)) != cudaSuccess) return cuda_fail(ce, "scratch A");
    int rc = repack_colmajor(g.a, g.m, g.k, 4, scratch[0], ld, s);
    if (rc) return rc;
    g.a = DevMat{scratch[0], 1, ld};
  }
  if (!unit(g.b, g.k, g.n)) {
    int64_t ld = round_up(g.k, 4);
    if ((ce = scratch_alloc(&scratch[1], (size_t)ld * g.n * 4, s)) != cudaSuccess) return cuda_fail(ce, "scratch B");
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
  p.o = Operands{static_cast<const float*>(g.a.ptr), g.a.rs, g.a.cs, static_cast<const float*>(g.b.ptr), g.b.rs,
                 g.b.cs, g.m, g.n, g.k, a_xc, b_xc, vec};
  p.e = Epi{g.m, g.n, (float)g.alpha, (float)g.beta, static_cast<float*>(g.c.ptr), g.c.rs, g.c.cs};
  // the tile and split count of this shape (tuning table or model)
  const PlainCfg cfg = plain_cfg(MOMMS_DTYPE_F32, g.m, g.n, g.k, ds->sm_count);
  const int TMv = cfg.tile == 1 ? 64 : 128;
  const int tiles_m = (int)ceil_div(g.m, TMv), tiles_n = (int)ceil_div(g.n, TMv);
  const int64_t tiles = (int64_t)tiles_m * tiles_n;
  const int64_t kblocks = ceil_div(g.k, BK);
  const int slots = ds->sm_count * (cfg.tile == 1 ? Tile<64>::CTAS_PER_SM : Tile<128>::CTAS_PER_SM);
  int splits = cfg.splits;
  int64_t kb_split = ceil_div(kblocks, splits);
  splits = (int)ceil_div(kblocks, kb_split);
  p.sched = TileSched{tiles_m, tiles_n, splits, 8, kb_split * BK};
  call_info().splits = splits;
  p.partials = nullptr;
  p.counters = nullptr;
  void*& ws = scratch[2];
  if (splits > 1) {
    size_t part_bytes = (size_t)tiles * splits * TMv * TMv * 4;
    size_t cnt_bytes = (size_t)tiles * 4;
    if ((ce = scratch_alloc(&ws, part_bytes + cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "split-k workspace");
    p.partials = static_cast<float*>(ws);
    p.counters = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + part_bytes);
    if ((ce = cudaMemsetAsync(p.counters, 0, cnt_bytes, s)) != cudaSuccess) return cuda_fail(ce, "memset counters");
  }
  const int grid = (int)std::min<int64_t>(p.sched.units(), slots);
  {
    KernelTimer kt(MOMMS_KERNEL_SGEMM_FFMA, s);
    // one instantiation per (tile, A layout, B layout, offset width, split)
    const int li = offsets_fit_32(p.o) ? 0 : 1, si = splits > 1 ? 1 : 0;
    if (cfg.tile == 1)
      kernel_table<64>()[a_xc][b_xc][li][si]<<<grid, Tile<64>::THREADS, Tile<64>::SMEM_BYTES, s>>>(p);
    else
      kernel_table<128>()[a_xc][b_xc][li][si]<<<grid, Tile<128>::THREADS, Tile<128>::SMEM_BYTES, s>>>(p);
  }
  note_launch();
  ce = launch_status();
  if (ce != cudaSuccess) return cuda_fail(ce, "sgemm_ffma launch");
  return MOMMS_OK;
}
}  // namespace

int launch_sgemm_ffma(const DevGemm& g, cudaStream_t s) {
  void* scratch[3] = {nullptr, nullptr, nullptr};
  const int rc = sgemm_ffma_impl(g, s, scratch);
  for (void* q : scratch)
    if (q) cudaFreeAsync(q, s);
  return rc;
}

}  // namespace momms
