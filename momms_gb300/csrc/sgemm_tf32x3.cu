// f32 GEMM as an error-compensated 3-term split-TF32 product on tcgen05.
//
// Each operand is split once into two TF32 planes, x = hi + lo with
// hi = tf32_rna(x) and lo = tf32_rna(x - hi) (the subtraction is exact), and
// C = beta*C + alpha*(A_lo B_hi + A_hi B_lo + A_hi B_hi) is accumulated in one
// FP32 TMEM accumulator (the dropped A_lo B_lo term is below 2^-22 relative;
// Markidis et al. 2018, Ootomo & Yokota 2022). The small cross terms are
// accumulated first. The result stays inside the f32 componentwise bound
// |dC| <= 2k u_32 (|A||B|) that the plain FFMA path meets.
#include "internal.h"
#include "planes.cuh"
#include "slicegemm.cuh"

namespace momms {

namespace {
struct Tf32SplitOp {
  static constexpr int PLANES = 2;  // hi, lo
  using Tout = float;
  using Word = uint2;  // one pair's float2 bits
  __device__ __forceinline__ int row(int64_t) const { return 0; }
  __device__ __forceinline__ static void split(float v, float* hi_out, float* lo_out) {
    uint32_t hi, lo;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(v));
    const float rest = v - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(rest));
    *hi_out = __uint_as_float(hi);
    *lo_out = __uint_as_float(lo);
  }
  // two neighbouring elements of a row: their hi pair and lo pair
  __device__ __forceinline__ void pack(float v0, float v1, int, uint2 (&out)[2]) const {
    float h0, h1, l0, l1;
    split(v0, &h0, &l0);
    split(v1, &h1, &l1);
    out[0] = make_uint2(__float_as_uint(h0), __float_as_uint(h1));
    out[1] = make_uint2(__float_as_uint(l0), __float_as_uint(l1));
  }
};
}  // namespace

int set_attrs_tf32() {
  cudaError_t e = sp::set_slice_attrs<1, sp::EPI_F32>();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "cudaFuncSetAttribute(split-TF32)");
}

void tf32_operand_planes(const float* x, int64_t sr, int64_t sp, int64_t R, int64_t K, float* planes, int64_t kp,
                         cudaStream_t s) {
  KernelTimer kt(MOMMS_KERNEL_PREP, s);
  planes::launch_to_planes(x, sr, sp, R, K, planes, kp, R * kp, Tf32SplitOp{}, s);
  note_launch();
}

int launch_sgemm_tf32x3(const DevGemm& g, cudaStream_t s) {
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  const int64_t kp = round_up(g.k, 4);  // 16-byte rows for TMA
  const size_t a_plane = (size_t)g.m * kp, b_plane = (size_t)g.n * kp;
  // packed operands (momms_pack) bring their planes
  const PackedOperand* PA = g.pk[0];
  const PackedOperand* PB = g.pk[1];
  void* buf = nullptr;
  cudaError_t ce = cudaSuccess;
  const size_t own = (PA ? 0 : 2 * a_plane) + (PB ? 0 : 2 * b_plane);
  if (own && (ce = scratch_alloc(&buf, own * sizeof(float), s)) != cudaSuccess)
    return cuda_fail(ce, "split-TF32 planes");
  ScratchGuard free_buf(buf, s);
  float* pa = PA ? static_cast<float*>(PA->planes) : static_cast<float*>(buf);
  float* pb = PB ? static_cast<float*>(PB->planes) : static_cast<float*>(buf) + (PA ? 0 : 2 * a_plane);
  // each operand's split waits only for that operand
  if (!PA) {
    if ((ce = wait_operand(g, 0, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
    tf32_operand_planes(static_cast<const float*>(g.a.ptr), g.a.rs, g.a.cs, g.m, g.k, pa, kp, s);
  }
  if (!PB) {
    if ((ce = wait_operand(g, 1, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
    tf32_operand_planes(static_cast<const float*>(g.b.ptr), g.b.cs, g.b.rs, g.n, g.k, pb, kp, s);
  }

  CUtensorMap tmA, tmB, tmB_half;
  {
    uint64_t dims[3] = {(uint64_t)g.k, (uint64_t)g.m, 2};
    uint64_t strides[2] = {(uint64_t)kp * 4, (uint64_t)a_plane * 4};
    uint32_t box[3] = {32, (uint32_t)sp::BM, 1};  // 128-byte k-blocks
    int rc = encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, pa, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    uint64_t dimsb[3] = {(uint64_t)g.k, (uint64_t)g.n, 2};
    uint64_t stridesb[2] = {(uint64_t)kp * 4, (uint64_t)b_plane * 4};
    uint32_t boxb[3] = {32, (uint32_t)sp::BN, 1};
    rc = encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, pb, dimsb, stridesb, boxb, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
    uint32_t boxh[3] = {32, (uint32_t)(sp::BN / 2), 1};  // one CTA's half of the B tile for the pair kernel
    rc = encode_tiled(&tmB_half, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, pb, dimsb, stridesb, boxh,
                      CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
  }

  sp::Params p;
  memset(&p, 0, sizeof(p));
  p.m = g.m;
  p.n = g.n;
  p.kelems = 32;
  p.kblocks = (int)ceil_div(g.k, 32);
  p.tiles_m = (int)ceil_div(g.m, sp::BM);
  p.tiles_n = (int)ceil_div(g.n, sp::BN);
  p.ngroups = 1;
  p.group_begin[0] = 0;
  p.group_begin[1] = 3;
  // small cross terms first, then hi*hi
  p.pair_a[0] = 1; p.pair_b[0] = 0;  // A_lo * B_hi
  p.pair_a[1] = 0; p.pair_b[1] = 1;  // A_hi * B_lo
  p.pair_a[2] = 0; p.pair_b[2] = 0;  // A_hi * B_hi
  // 256 k per tensor-core accumulation (8 k-blocks of one pair), then an RN
  // add in registers; chunks never span pairs
  for (int i = 0; i < 3; ++i) p.pair_w[i] = 1;
  p.chunk_cap = 8;
  p.merge_pairs = 0;
  p.alpha_f = (float)g.alpha;
  p.beta_f = (float)g.beta;
  p.c32 = static_cast<float*>(g.c.ptr);
  p.rsc = g.c.rs;
  p.csc = g.c.cs;
  p.status = ds->status;

  // the epilogue reads C
  if ((ce = wait_operand(g, 2, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
  {
    KernelTimer kt(MOMMS_KERNEL_SLICE_TF32, s);
    int variant = 0;
    ce = sp::launch_slice<1, sp::EPI_F32>(tmA, tmB, tmB_half, p, ds->sm_count, s, &variant);
    if (ce != cudaSuccess) return cuda_fail(ce, "split-TF32 slice launch");
    call_info().slice_variant = variant;
  }
  note_launch();
  ce = launch_status();
  if (ce != cudaSuccess) return cuda_fail(ce, "split-TF32 launch");
  return MOMMS_OK;
}

}  // namespace momms
