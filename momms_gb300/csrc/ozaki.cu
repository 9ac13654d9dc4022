// FP64 GEMM emulated on the fp16 tensor cores (Ozaki scheme, slice products).
//
// Ozaki, Ogita, Oishi, Rump (2012): scale each row of A (column of B) by a
// power of two so that its entries lie in (-1, 1), split every scaled entry
// into s signed digits of `bits` bits,
//     x = 2^e * sum_{t=1..s} d_t 2^(-bits*t),   d_t integers, |d_t| <= 2^bits,
// and form A*B from digit-plane products A_t * B_u, each exact in a
// wide-enough accumulator. Products on the same anti-diagonal d = t + u share
// the weight 2^(-bits*d); the scheme keeps d <= s + 1 (triangular truncation).
//
// GB300 form (sm_103a has no integer tcgen05 kind): digits are 8-bit integers
// held as fp16 values (exact for |d| <= 2048), the products run on tcgen05
// kind::f16 with FP32 accumulation in TMEM, and every accumulation chunk's
// sum of absolute products is kept at or below 2^24, so that every partial
// sum is an exactly representable integer; chunks are gathered in int32
// registers, and the diagonals are combined exactly (64-bit partial sums per
// 32-bit word offset, up to 148 bits) and rounded once to FP64
// (exact_round.cuh). See slicegemm.cuh for the engine. With 8-bit digits 7 slices cover 56 bits with
// 28 slice products, where 7-bit digits need 8 slices and 36 products; the
// price is 4x larger products, so TMEM is drained every 4 (top x top), 8 (top
// x centred) or 16 (centred x centred) k-blocks.
//
// The slice count is chosen per call from the requested componentwise error
// (|dC_ij| / (|A||B|)_ij): with RN digits the truncation error is at most
//   2^(-bits*s-1) * (2^e_i sum_p |b_pj| + 2^f_j sum_p |a_ip|
//                    + (s-1)/2 * k * 2^(e_i+f_j))
// (digit truncation of A and B, then the largest dropped diagonal), and the
// bound kernel bounds (|A||B|)_ij from below for every entry, so the count
// holds for every entry of C (a sampled estimate starts host-staged calls
// early; the bound then verifies it before C is written).
#include <cuda_fp16.h>
#include <math.h>
#include <stdlib.h>

#include <algorithm>
#include <type_traits>

#include "internal.h"
#include "exact_round.cuh"
#include "ozaki_elem.cuh"
#include "planes.cuh"
#include "slicegemm.cuh"

namespace momms {
namespace {

constexpr int kDigitBits = elem::kDigitBits;
using elem::abs_bits;
using elem::exponent_of_max;
using elem::magnitude;
using elem::offset_digits;
// k per launch (kOzakiMaxK): the largest product of two digits is 2^16, so a
// single pair's int32 sum stays below 2^31 for up to 511 k-blocks of 64
constexpr int64_t kMaxK = kOzakiMaxK;
static_assert((kMaxK / 64) * 64 * (1ll << (2 * kDigitBits)) < (1ll << 31), "int32 digit sums must stay exact");
// an int32 group sum's bound (sums of the pairs' worst cases)
constexpr double kGroupLimit = 2147483647.0;
// one TMEM chunk's bound: integers up to 2^24 are exact in FP32
constexpr double kChunkBound = 16777216.0;

// Everything in the pre-pass runs on integer bit patterns: GB300's FP64 pipe
// is about 1 TFLOP/s, so FP64 arithmetic per element would dominate.

// Row maxima of |x(r, p)| as bit patterns, rows contiguous (sr == 1, a
// column-major A). A block covers 32 rows x 256 of p: lanes along r, the 8
// warps striding over p, each thread's 32 loads issued before the first
// maximum; the warps' maxima meet in shared memory and one atomicMax per row
// posts them (maxbits must start at zero). At 8192^2 this reads at 5.0 TB/s
// (104-108 us), against 4.0 for the run layout of the other prep kernels
// (133 us); with p contiguous the run layout is the faster one (132 us,
// against 230 for a warp per row with lanes along p in this block shape).
__global__ void __launch_bounds__(256) row_absmax_kernel(const double* __restrict__ x, int64_t sp, int64_t R,
                                                         int64_t K, unsigned long long* __restrict__ maxbits) {
  __shared__ unsigned long long red[8][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t r = (int64_t)blockIdx.y * 32 + tx, p0 = (int64_t)blockIdx.x * 256;
  unsigned long long mx = 0;
  if (r < R) {
    double v[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int64_t pp = p0 + ty + 8 * j;
      v[j] = pp < K ? x[r + pp * sp] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) mx = max(mx, abs_bits(v[j]));
  }
  red[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && r < R) {
    for (int i = 1; i < 8; ++i) mx = max(mx, red[i][tx]);
    if (mx) atomicMax(&maxbits[r], mx);
  }
}

// Row maxima with p contiguous (or general strides), in the run layout of
// planes.cuh: the lanes of one row reduce by shuffles and one posts an
// atomicMax (maxbits must start at zero).
__global__ void __launch_bounds__(planes::THREADS)
    row_absmax_runs_kernel(const double* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K, bool vec,
                           int lg, unsigned long long* __restrict__ maxbits) {
  constexpr int RUN = 8;
  const planes::Chunk<false> c(lg);
  // the row loop's trip count is the same for every thread of the block, so
  // every lane reaches the shuffles
  for (int64_t rb = (int64_t)blockIdx.y * c.rows; rb < R; rb += (int64_t)gridDim.y * c.rows) {
    const int64_t r = rb + c.rl;
    unsigned long long mx = 0;
    if (r < R) {
      const double* xr = x + r * sr;
#pragma unroll 1
      for (int it = 0; it < planes::PITER; ++it) {
        const int64_t p = planes::run_col(blockIdx.x, c, it, RUN);
        if (p >= K) break;
        double v[RUN];
        planes::load_run<false, RUN>(xr, sp, p, K, vec, v);
#pragma unroll
        for (int i = 0; i < RUN; ++i) mx = max(mx, abs_bits(v[i]));
      }
    }
    for (int o = c.runs >> 1; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (c.ru == 0 && r < R && mx) atomicMax(&maxbits[r], mx);
  }
}

__global__ void exps_kernel(const unsigned long long* __restrict__ maxbits, int64_t count, int* __restrict__ exps) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  exps[i] = exponent_of_max(maxbits[i]);
}

// Digit planes of an operand for NS slices: plane t holds digit position
// NS-1-t of every element (plane 0 the top digit), sign applied, as fp16.
// A pair of digits d0, d1 in [-2^bits, 2^bits] becomes one __half2 without a
// conversion instruction: the fp16 bit patterns 0x6400 + u are the integers
// 1024 + u (u < 1024), so packing u = d + 2^bits under 0x6400 and subtracting
// 1024 + 2^bits gives d exactly (and +0 for d = 0, as an integer conversion
// does).
template <int NS>
struct OzakiSliceOp {
  static constexpr int PLANES = NS;
  using Tout = __half;
  using Word = uint32_t;  // one pair's __half2 bits
  using U = typename std::conditional<(kDigitBits * NS <= 62), unsigned long long, unsigned __int128>::type;
  const int* exps;
  __device__ __forceinline__ int row(int64_t r) const { return exps[r]; }
  // 32-bit word w of Y
  __device__ __forceinline__ static uint32_t word(U y, int w) { return (uint32_t)(y >> (32 * w)); }
  __device__ __forceinline__ static uint32_t bits_of(__half2 h) { return *reinterpret_cast<const uint32_t*>(&h); }
  __device__ __forceinline__ void pack(double v0, double v1, int e, uint32_t (&out)[NS]) const {
    constexpr int bits = kDigitBits;
    static_assert(bits == 8, "lower digits are the bytes of Y");
    const U Y0 = offset_digits<NS, U>(v0, e), Y1 = offset_digits<NS, U>(v1, e);
    const bool n0 = __double_as_longlong(v0) < 0, n1 = __double_as_longlong(v1) < 0;
    static_assert(2 * (1 << bits) < 1024, "digits must fit the 0x6400 pattern");
    constexpr unsigned short kBias = 0x6400 + (1u << bits);  // 1024 + 2^bits
    const __half2 bias = __halves2half2(__ushort_as_half(kBias), __ushort_as_half(kBias));
    // A lower digit d = byte - 2^(bits-1) of a value of sign n is held as
    // u = (n ? -d : d) + 2^bits, that is byte + 128 or (byte ^ 0xff) + 129:
    // for both elements of the pair at once, bytes in 16-bit lanes 0 and 1.
    const uint32_t flip = (n0 ? 0xffu : 0u) | (n1 ? 0xff0000u : 0u);
    const uint32_t add = 0x64006400u + ((n0 ? 129u : 128u) | ((n1 ? 129u : 128u) << 16));
    // digit position pos goes to plane NS-1-pos
#pragma unroll
    for (int pos = 0; pos < NS - 1; ++pos) {
      const uint32_t b = __byte_perm(word(Y0, pos >> 2), word(Y1, pos >> 2), (pos & 3) | ((4 + (pos & 3)) << 8));
      const uint32_t w = ((b & 0x00ff00ffu) ^ flip) + add;
      out[NS - 1 - pos] = bits_of(__hsub2(*reinterpret_cast<const __half2*>(&w), bias));
    }
    {
      // top digit: the remaining bits, in [0, 2^bits]
      const int d0 = (int)(unsigned)(Y0 >> (bits * (NS - 1))), d1 = (int)(unsigned)(Y1 >> (bits * (NS - 1)));
      const unsigned u0 = (unsigned)((n0 ? -d0 : d0) + (1 << bits)), u1 = (unsigned)((n1 ? -d1 : d1) + (1 << bits));
      const unsigned w = 0x64006400u | u0 | (u1 << 16);
      out[0] = bits_of(__hsub2(*reinterpret_cast<const __half2*>(&w), bias));
    }
  }
};

template <int NS>
void launch_ozaki_planes(const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K, __half* planes, int64_t ldp,
                         int64_t plane_elems, const int* exps, cudaStream_t s) {
  planes::launch_to_planes(x, sr, sp, R, K, planes, ldp, plane_elems, OzakiSliceOp<NS>{exps}, s);
}

// Runtime slice count -> the unrolled kernel for it (1..kOzakiMaxSlices).
void ozaki_planes(int ns, const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K, __half* planes, int64_t ldp,
                  int64_t plane_elems, const int* exps, cudaStream_t s) {
  switch (ns) {
#define MOMMS_OZAKI_NS(N) \
  case N: launch_ozaki_planes<N>(x, sr, sp, R, K, planes, ldp, plane_elems, exps, s); break;
    MOMMS_OZAKI_NS(1) MOMMS_OZAKI_NS(2) MOMMS_OZAKI_NS(3) MOMMS_OZAKI_NS(4) MOMMS_OZAKI_NS(5) MOMMS_OZAKI_NS(6)
    MOMMS_OZAKI_NS(7) MOMMS_OZAKI_NS(8) MOMMS_OZAKI_NS(9) MOMMS_OZAKI_NS(10) MOMMS_OZAKI_NS(11) MOMMS_OZAKI_NS(12)
    MOMMS_OZAKI_NS(13) MOMMS_OZAKI_NS(14) MOMMS_OZAKI_NS(15)
#undef MOMMS_OZAKI_NS
    default: break;
  }
}

// Sampled quantities for the slice-count bound: for sampled (i, j),
//   q1 = (2^e_i sum|b_.j| + 2^f_j sum|a_i.|) / (|A||B|)_ij
//      = (sum b' + sum a') / sum a'b'
//   q2 = k 2^(e_i+f_j) / (|A||B|)_ij = k / sum a'b'
// with a' = |a| 2^-e_i and b' = |b| 2^-f_j in [0, 1), reduced to their maxima
// in out[0], out[1] (as ordered non-negative floats). The scaled magnitudes
// are built from the exponent bits as FP32 (mantissa truncated, below 2^-126
// flushed: an estimate needs no more), so the sums run on the FP32 pipe
// rather than GB300's narrow FP64 one.
// Sample (x, y) is 32 consecutive rows of A against one column of B, at
// hashed positions. The sums run in two steps so that the work spreads over
// the GPU and the result does not depend on timing: sample_partial_kernel
// block (x, y, z) sums k range z (lanes walk the rows, coalesced for
// column-major A; warps split the range) into its own slot, and
// sample_final_kernel adds the slots in a fixed order.
constexpr int kSampleRowBlocks = 8, kSampleCols = 8, kSamples = kSampleRowBlocks * kSampleCols;
constexpr int kSampleSlot = 2 * 32 + 1;  // sab[32], sa[32], sb

__host__ __device__ __forceinline__ void sample_position(int x, int y, int64_t m, int64_t n, int64_t* i0,
                                                         int64_t* j) {
  uint64_t h = 0x9E3779B97F4A7C15ull * (uint64_t)(x * 131 + y * 7 + 1);
  h ^= h >> 31;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 29;
  *i0 = m > 32 ? (int64_t)(h % (uint64_t)(m - 31)) : 0;
  *j = (int64_t)((h >> 24) % (uint64_t)n);
}

// |v| * 2^-e as FP32 from the bit pattern (|v| < 2^e, so at most just below 1).
__device__ __forceinline__ float scaled_abs(double v, int e) {
  const unsigned long long ab = abs_bits(v);
  const int be = (int)(ab >> 52);
  const int fe = be - 1023 - e + 127;
  if (e == INT32_MAX || be == 0 || fe <= 0) return 0.0f;
  return __uint_as_float(((unsigned)fe << 23) | (unsigned)((ab >> 29) & 0x7fffffull));
}

__global__ void __launch_bounds__(256) sample_partial_kernel(const double* __restrict__ a, int64_t rsa, int64_t csa,
                                                             const double* __restrict__ b, int64_t rsb, int64_t csb,
                                                             int64_t m, int64_t n, int64_t k, int64_t kc,
                                                             const int* __restrict__ rexp,
                                                             const int* __restrict__ cexp, double* __restrict__ part) {
  __shared__ double s_ab[8][32], s_a[8][32], s_b[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t i0, j;
  sample_position(blockIdx.x, blockIdx.y, m, n, &i0, &j);
  const int64_t i = i0 + lane;
  const int ei = i < m ? rexp[i] : 0, fj = cexp[j];
  const int64_t k0 = (int64_t)blockIdx.z * kc, k1 = min(k, k0 + kc);
  float sab = 0.0f, sa = 0.0f, sb = 0.0f;
  for (int64_t pp = k0 + warp; pp < k1; pp += 8) {
    const float bv = scaled_abs(b[pp * rsb + j * csb], fj);
    sb += bv;
    if (i < m) {
      const float av = scaled_abs(a[i * rsa + pp * csa], ei);
      sab = fmaf(av, bv, sab);
      sa += av;
    }
  }
  s_ab[warp][lane] = sab;
  s_a[warp][lane] = sa;
  if (lane == 0) s_b[warp] = sb;
  __syncthreads();
  if (warp == 0) {
    double tab = 0.0, ta = 0.0;
    for (int w = 0; w < 8; ++w) {
      tab += s_ab[w][lane];
      ta += s_a[w][lane];
    }
    double* slot = part + ((int64_t)blockIdx.z * kSamples + blockIdx.y * kSampleRowBlocks + blockIdx.x) * kSampleSlot;
    slot[lane] = tab;
    slot[32 + lane] = ta;
    if (lane == 0) {
      double t = 0.0;
      for (int w = 0; w < 8; ++w) t += s_b[w];
      slot[64] = t;
    }
  }
}

// Column exponents of B at the sampled columns only (the same values the
// per-column scan gives), so that the slice count can be chosen before the
// rest of B is on the device. Samples sharing a column write the same value.
__global__ void __launch_bounds__(256) sample_col_exps_kernel(const double* __restrict__ b, int64_t rsb, int64_t csb,
                                                              int64_t m, int64_t n, int64_t k,
                                                              int* __restrict__ cexp) {
  __shared__ unsigned long long red[8];
  int64_t i0, j;
  sample_position(blockIdx.x % kSampleRowBlocks, blockIdx.x / kSampleRowBlocks, m, n, &i0, &j);
  unsigned long long mx = 0;
  for (int64_t pp = threadIdx.x; pp < k; pp += 256) mx = max(mx, abs_bits(b[pp * rsb + j * csb]));
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < 8; ++w) mx = max(mx, red[w]);
    cexp[j] = exponent_of_max(mx);
  }
}

// One warp per sample: adds the k-range slots in order, then the maxima.
__global__ void __launch_bounds__(32) sample_final_kernel(const double* __restrict__ part, int nz, int64_t m,
                                                          int64_t n, int64_t k, const int* __restrict__ rexp,
                                                          const int* __restrict__ cexp, unsigned long long* out) {
  const int lane = threadIdx.x;
  const int x = blockIdx.x % kSampleRowBlocks, y = blockIdx.x / kSampleRowBlocks;
  int64_t i0, j;
  sample_position(x, y, m, n, &i0, &j);
  const int64_t i = i0 + lane;
  double sab = 0.0, sa = 0.0, sb = 0.0;
  for (int z = 0; z < nz; ++z) {
    const double* slot = part + ((int64_t)z * kSamples + blockIdx.x) * kSampleSlot;
    sab += slot[lane];
    sa += slot[32 + lane];
    sb += slot[64];
  }
  if (i >= m) return;
  const int ei = rexp[i], fj = cexp[j];
  if (ei == INT32_MAX || fj == INT32_MAX || sab == 0.0) return;
  const double q1 = (sb + sa) / sab;
  const double q2 = (double)k / sab;
  // non-negative doubles order like their bit patterns
  atomicMax(&out[0], (unsigned long long)__double_as_longlong(q1));
  atomicMax(&out[1], (unsigned long long)__double_as_longlong(q2));
}

// Recombination of the exact group sums. Group g holds S_g = the int32 sum of
// the digit products of diagonal d_g (weight 2^(-bits*(d_g-2))), so
//   R = sum_g S_g * 2^(bits*(dmax - (d_g-2)))
// is an exact integer (below 2^(31 + bits*dmax + 3): 2^147 at 15 slices), and
//   C = beta*C + alpha * 2^(e_i + f_j - 2 bits - bits*dmax) * R
// with R rounded to double once. All the summation is integer arithmetic;
// FP64 is used for the final conversion, scaling and beta update only.
//
// R is formed from 64-bit partial sums, one per 32-bit word offset (four at
// 13-15 slices, three below): group g's weight 2^sh (sh = bits*(dmax -
// level) <= 112) is split into a word gw[g] = sh / 32 and a shift
// gb[g] = sh % 32 <= 24, so that R = P0 + P1 2^32 + P2 2^64 + P3 2^96 with
// P_w = sum over the groups of word w of S_g 2^gb[g]: each term is below 2^55
// and a word holds at most four levels (at most eight groups each), so no
// partial sum leaves 64 bits. Every level enters exactly, up to the most
// slices (dmax = 14), and R is rounded once (i128_to_double / wide_to_double,
// exact_round.cuh).
struct CombineParams {
  const int* sbuf;  // tile-blocked group planes (sp::Params::sbuf)
  int64_t plane;
  int64_t mpad;     // m rounded up to the slice kernel's tile height
  int ng;
  uint8_t gw[sp::MAX_GROUPS];  // word offset of group g (0..3)
  uint8_t gb[sp::MAX_GROUPS];  // left shift within the word
  int scale_off;  // -2 bits - bits*dmax
  int alpha_one, beta_zero;
  int wide;  // some group has word 3 (13-15 slices): R may pass 2^127 (wide_to_double)
  int levels;  // > 0: group g has weight 2^(bits g) for g < levels = ng (combine_kernel's fixed form)
  int64_t m;
  int64_t j0, j1;  // columns of C this launch finishes
  const int* row_exp;
  const int* col_exp;
  double alpha, beta;
  double* c;
  int64_t rsc, csc;
};

// Thread rows i and i + 256 of block row blockIdx.x, for columns
// j0 + blockIdx.y, stepping by gridDim.y: no index division, the row
// exponents stay in registers, and the two rows' loads are in flight together.
//
// The forms, one integer R:
//  * NS > 0: one group per level (every k up to 8192), so group g's weight
//    is 2^(bits g) and every word offset and shift is a compile-time
//    constant: one 32 x 32 + 64-bit multiply-add per group and row;
//  * NS == 0: any grouping, the weights read per group;
//  * WIDE: 13-15 slices (a fourth partial sum and the conversion from up to
//    148 bits), NARROW up to 12.
// The kernel is bound by its issue rate and its memory latency together, so
// the narrow forms keep to 64 registers (four blocks per SM). At 4096 x 4096
// x 64 with 7 slices the runtime-weight form issued 332 instructions per
// entry (ALU pipe 48 %, DRAM 30 % of peak, 298 us); the fixed form with
// shift-and-add sums 194 (ALU 70 %, DRAM 65 %, 140 us).
template <bool WIDE, int NS>
__global__ void __launch_bounds__(256, WIDE ? 2 : 4) combine_kernel(const __grid_constant__ CombineParams p) {
  static_assert(NS == 0 || (NS * kDigitBits <= 96) != WIDE, "the wide form is for levels past word 2");
  using u128 = unsigned __int128;
  constexpr int NW = WIDE ? 4 : 3;
  // group sums whose loads are issued together: NS, else every group of up
  // to 8 (narrow) or 16 (wide) groups
  constexpr int kBatch = NS > 0 ? NS : (WIDE ? 16 : 8);
  int64_t rows[2], roff[2];
  int er[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    rows[u] = (int64_t)blockIdx.x * 512 + threadIdx.x + 256 * u;
    er[u] = rows[u] < p.m ? p.row_exp[rows[u]] : 0;
    roff[u] = (rows[u] / sp::BM) * (sp::BM * sp::BN) + rows[u] % sp::BM;  // row's place in the tile blocks
  }
  if (rows[0] >= p.m) return;
  const bool two = rows[1] < p.m;
  for (int64_t j = p.j0 + blockIdx.y; j < p.j1; j += gridDim.y) {
    const int ec = p.col_exp[j];
    const int* col = p.sbuf + (j / sp::BN) * (p.mpad * sp::BN) + (j % sp::BN) * sp::BM;
    // C's old values are loaded with the group sums, not after the sums, so
    // a column costs one memory round trip
    double c_old[2] = {0.0, 0.0};
    if (!p.beta_zero) {
      c_old[0] = p.c[rows[0] * p.rsc + j * p.csc];
      if (two) c_old[1] = p.c[rows[1] * p.rsc + j * p.csc];
    }
    // the 64-bit partial sums of each of the two rows (see CombineParams)
    long long P[NW][2];
#pragma unroll
    for (int w = 0; w < NW; ++w) P[w][0] = P[w][1] = 0;
    auto add = [&](int u, int s_g, int g) {
      const int w = p.gw[g], f = 1 << p.gb[g];  // gb <= 24
      if (w == 0) {
        P[0][u] = mad_wide(s_g, f, P[0][u]);
      } else if (w == 1) {
        P[1][u] = mad_wide(s_g, f, P[1][u]);
      } else if constexpr (WIDE) {
        if (w == 2) P[2][u] = mad_wide(s_g, f, P[2][u]);
        else P[NW - 1][u] = mad_wide(s_g, f, P[NW - 1][u]);
      } else {
        P[2][u] = mad_wide(s_g, f, P[2][u]);
      }
    };
    if (NS > 0 || p.ng <= kBatch) {
      // all loads first (up to 2 x kBatch in flight), then the sums
      int s0[kBatch], s1[kBatch];
#pragma unroll
      for (int q = 0; q < kBatch; ++q) {
        s0[q] = 0;
        s1[q] = 0;
        if (NS > 0 || q < p.ng) {
          const int* sg = col + (int64_t)q * p.plane;
          s0[q] = sg[roff[0]];
          if (two) s1[q] = sg[roff[1]];
        }
      }
#pragma unroll
      for (int q = 0; q < kBatch; ++q) {
        if constexpr (NS > 0) {
          // weight 2^(bits q): word (bits q) / 32, shift (bits q) % 32, both
          // constants once the loop is unrolled
          constexpr int bits = kDigitBits;
          P[(bits * q) >> 5][0] = mad_wide(s0[q], 1 << ((bits * q) & 31), P[(bits * q) >> 5][0]);
          P[(bits * q) >> 5][1] = mad_wide(s1[q], 1 << ((bits * q) & 31), P[(bits * q) >> 5][1]);
        } else if (q < p.ng) {
          add(0, s0[q], q);
          add(1, s1[q], q);
        }
      }
    } else {
      for (int q = 0; q < p.ng; ++q) {
        const int* sg = col + (int64_t)q * p.plane;
        add(0, sg[roff[0]], q);
        if (two) add(1, sg[roff[1]], q);
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      if (u == 1 && !two) break;
      double v;
      const int sc = er[u] + ec + p.scale_off;
      if (er[u] == INT32_MAX || ec == INT32_MAX) {
        v = __longlong_as_double(0x7ff8000000000000ll);
      } else if constexpr (WIDE) {
        v = wide_to_double(P[0][u], P[1][u], P[2][u], P[NW - 1][u], sc);
      } else {
        // |R| < 2^127: 128-bit two's complement holds it
        const u128 R = (u128)(__int128)P[0][u] + ((u128)(__int128)P[1][u] << 32) + ((u128)(__int128)P[2][u] << 64);
        v = i128_to_double((__int128)R, sc);
      }
      double* cp = p.c + rows[u] * p.rsc + j * p.csc;
      const double sv = p.alpha_one ? v : v * p.alpha;  // v * 1 == v: one FP64 operation saved
      *cp = p.beta_zero ? sv : fma(p.beta, c_old[u], sv);
    }
  }
}

// Worst-case componentwise error of an s-slice product, relative to |A||B|.
double ozaki_bound(int s, int bits, double q1, double q2) {
  return ldexp(1.0, -bits * s - 1) * (q1 + 0.5 * (s - 1) * q2);
}

// Row exponents of A (first m) and column exponents of B (next n).
int compute_exponents(const DevGemm& g, unsigned long long* maxbits, int* exps, cudaStream_t s) {
  // A viewed as m x k; B viewed transposed, n x k
  int rc = ozaki_operand_exponents(static_cast<const double*>(g.a.ptr), g.a.rs, g.a.cs, g.m, g.k, maxbits, exps, s);
  if (!rc)
    rc = ozaki_operand_exponents(static_cast<const double*>(g.b.ptr), g.b.cs, g.b.rs, g.n, g.k, maxbits + g.m,
                                 exps + g.m, s);
  return rc;
}

// Smallest slice count whose sampled worst-case bound meets the target
// (0 = FP64 level, 2^-52). Synchronises the stream once to read the sample.
int choose_slices(const DevGemm& g, const int* rexp, const int* cexp, double target, int bits, cudaStream_t s,
                  int* ns_out, double* bound_out) {
  const double tgt = target > 0.0 ? target : ldexp(1.0, -52);
  // k ranges of at least 512 per block, at most 32 ranges
  const int nz = (int)std::max<int64_t>(1, std::min<int64_t>(32, g.k / 512));
  const int64_t kc = ceil_div(g.k, nz);
  unsigned long long* q = nullptr;
  const size_t part_bytes = (size_t)nz * kSamples * kSampleSlot * sizeof(double);
  cudaError_t ce = scratch_alloc(&q, 2 * sizeof(unsigned long long) + part_bytes, s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki bound sample");
  double* part = reinterpret_cast<double*>(q + 2);
  cudaMemsetAsync(q, 0, 2 * sizeof(unsigned long long), s);
  sample_partial_kernel<<<dim3(kSampleRowBlocks, kSampleCols, nz), 256, 0, s>>>(
      static_cast<const double*>(g.a.ptr), g.a.rs, g.a.cs, static_cast<const double*>(g.b.ptr), g.b.rs, g.b.cs, g.m,
      g.n, g.k, kc, rexp, cexp, part);
  sample_final_kernel<<<kSamples, 32, 0, s>>>(part, nz, g.m, g.n, g.k, rexp, cexp, q);
  note_launch(2);
  unsigned long long hq[2] = {0, 0};
  ce = cudaMemcpyAsync(hq, q, sizeof(hq), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  cudaFreeAsync(q, s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki bound sample");
  double q1, q2;
  memcpy(&q1, &hq[0], 8);
  memcpy(&q2, &hq[1], 8);
  if (!(q1 > 0.0)) q1 = 4.0;  // no usable sample (zero operands): nominal uniform-data value
  if (!(q2 > 0.0)) q2 = 4.0;
  int ns = 1;
  while (ns < kOzakiMaxSlices && ozaki_bound(ns, bits, q1, q2) > tgt) ++ns;
  *ns_out = ns;
  if (bound_out) *bound_out = ozaki_bound(ns, bits, q1, q2);
  return MOMMS_OK;
}

}  // namespace

int ozaki_operand_exponents(const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K,
                            unsigned long long* maxbits, int* exps, cudaStream_t s) {
  if (R == 0) return MOMMS_OK;
  const bool r_contig = (sr == 1 && sp != 1);
  KernelTimer kt(MOMMS_KERNEL_PREP, s);
  cudaError_t ce = cudaMemsetAsync(maxbits, 0, (size_t)R * sizeof(unsigned long long), s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki exponents");
  int launches = 1;
  if (r_contig) {
    // rows in launches of at most 65535 row tiles (the grid's y limit)
    for (int64_t rb = 0; rb < R; rb += (int64_t)65535 * 32, ++launches) {
      const int64_t rn = std::min<int64_t>(R - rb, (int64_t)65535 * 32);
      row_absmax_kernel<<<dim3((unsigned)ceil_div(K, 256), (unsigned)ceil_div(rn, 32)), dim3(32, 8), 0, s>>>(
          x + rb, sp, rn, K, maxbits + rb);
    }
  } else {
    const int lg = planes::run_lanes_log2(K, 8, false, planes::kRowsContigLg);
    row_absmax_runs_kernel<<<planes::run_grid<false, 8>(R, K, lg), planes::THREADS, 0, s>>>(
        x, sr, sp, R, K, planes::rows_vector_aligned(x, sr, sp), lg, maxbits);
    ++launches;
  }
  exps_kernel<<<(unsigned)ceil_div(R, 256), 256, 0, s>>>(maxbits, R, exps);
  note_launch(launches);
  ce = launch_status();
  return ce == cudaSuccess ? MOMMS_OK : cuda_fail(ce, "Ozaki exponents");
}

void ozaki_operand_planes(int ns, const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K, void* planes,
                          int64_t kp, const int* exps, cudaStream_t s) {
  KernelTimer kt(MOMMS_KERNEL_PREP, s);
  ozaki_planes(ns, x, sr, sp, R, K, static_cast<__half*>(planes), kp, R * kp, exps, s);
  note_launch();
}

int set_attrs_ozaki() {
  cudaError_t e = sp::set_slice_attrs<0, sp::EPI_OZAKI>();
  if (e == cudaSuccess) e = sp::set_slice_attrs<2, sp::EPI_BOUND>();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "cudaFuncSetAttribute(Ozaki)");
}

namespace {
// The slice-product schedule for ns slices over k: diagonals d = t + u from
// the smallest weight (d = ns+1) to the largest (d = 2), each diagonal's pairs
// (t, d-t) in t order, cut into accumulation groups whose worst-case int32
// sums (k * 2^bits_t * 2^bits_u over the group's pairs; the top digit has
// `bits` bits, the centred ones bits-1) stay within kGroupLimit. A group's
// A TMEM chunk keeps its sum within kChunkBound: a k-block of pair (t, u)
// adds at most 64 * 2^bits_t * 2^bits_u, so a pair's weight is that product
// in units of 2^10 and a chunk's capacity kChunkBound / 64 / 2^10 (a lone
// pair: 4, 8 or 16 k-blocks of 64 for 8-bit digits; at small k one chunk
// spans several pairs of a group).
constexpr int kChunkUnitLog2 = 10;
constexpr int kChunkCap = (int)(kChunkBound / 64.0) >> kChunkUnitLog2;
struct Schedule {
  int np = 0, ng = 0;
  uint8_t pair_a[sp::MAX_PAIRS], pair_b[sp::MAX_PAIRS];
  int group_begin[sp::MAX_GROUPS + 1];
  int pair_w[sp::MAX_PAIRS];
  uint8_t level[sp::MAX_GROUPS];  // d - 2
};

bool ozaki_schedule(int ns, int64_t k, Schedule* sc) {
  const int bits = kDigitBits;
  const int64_t kblocks = ceil_div(std::min<int64_t>(std::max<int64_t>(k, 1), kMaxK), 64);
  const double kspan = (double)kblocks * 64.0;
  auto prod = [&](int t, int u) { return ldexp(1.0, (t == 1 ? bits : bits - 1) + (u == 1 ? bits : bits - 1)); };
  sc->np = sc->ng = 0;
  for (int d = ns + 1; d >= 2; --d) {
    double gsum = 0.0;
    bool open = false;
    for (int t = 1; t <= ns; ++t) {
      const int u = d - t;
      if (u < 1 || u > ns) continue;
      const double pb = prod(t, u);
      if (open && gsum + kspan * pb > kGroupLimit) open = false;  // this pair starts the next group
      if (!open) {
        if (sc->ng >= sp::MAX_GROUPS) return false;
        sc->group_begin[sc->ng] = sc->np;
        sc->level[sc->ng] = (uint8_t)(d - 2);
        ++sc->ng;
        gsum = 0.0;
        open = true;
      }
      if (sc->np >= sp::MAX_PAIRS) return false;
      sc->pair_a[sc->np] = (uint8_t)(t - 1);
      sc->pair_b[sc->np] = (uint8_t)(u - 1);
      sc->pair_w[sc->np] = std::max(1, (int)ldexp(pb, -kChunkUnitLog2));
      ++sc->np;
      gsum += kspan * pb;
    }
  }
  sc->group_begin[sc->ng] = sc->np;
  return true;
}
}  // namespace

namespace {
// The slice kernel's parameters of an ns-slice product over k (rows m): the
// schedule's pairs and groups, the TMEM chunk rule. Sizes along n, the output
// planes and the status word are the caller's.
bool slice_params(int ns, int64_t m, int64_t k, sp::Params* p, Schedule* sch) {
  if (!ozaki_schedule(ns, k, sch)) return false;
  memset(p, 0, sizeof(*p));
  p->m = m;
  p->kelems = 64;
  p->kblocks = (int)ceil_div(k, 64);
  p->tiles_m = (int)ceil_div(m, sp::BM);
  const int np = sch->np, ng = sch->ng;
  memcpy(p->pair_a, sch->pair_a, (size_t)np);
  memcpy(p->pair_b, sch->pair_b, (size_t)np);
  memcpy(p->group_begin, sch->group_begin, sizeof(int) * (size_t)(ng + 1));
  memcpy(p->pair_w, sch->pair_w, sizeof(int) * (size_t)np);
  p->chunk_cap = kChunkCap;
  p->merge_pairs = 1;
  p->ngroups = ng;
  return true;
}

// The recombination's parameters for the whole of C (columns 0..n).
void combine_params(const DevGemm& g, int ns, const Schedule& sch, const int* sbuf, int64_t plane, int64_t mpad,
                    const int* rexp, const int* cexp, CombineParams* cp) {
  const int bits = kDigitBits;
  memset(cp, 0, sizeof(*cp));
  cp->sbuf = sbuf;
  cp->plane = plane;
  cp->mpad = mpad;
  // each group's weight 2^(bits*(dmax - level)) as (word, shift)
  const int dmax = ns - 1;
  cp->ng = sch.ng;
  for (int gi = 0; gi < sch.ng; ++gi) {
    const int sh = bits * (dmax - sch.level[gi]);
    cp->gw[gi] = (uint8_t)(sh >> 5);
    cp->gb[gi] = (uint8_t)(sh & 31);
    if (cp->gw[gi] == 3) cp->wide = 1;
  }
  // one group per level, lowest first: the weights are 2^(bits g)
  bool one_per_level = sch.ng <= kOzakiMaxSlices;
  for (int gi = 0; gi < sch.ng && one_per_level; ++gi) one_per_level = 32 * cp->gw[gi] + cp->gb[gi] == bits * gi;
  cp->levels = one_per_level ? sch.ng : 0;
  cp->scale_off = -2 * bits - bits * dmax;
  cp->alpha_one = (g.alpha == 1.0);
  cp->beta_zero = (g.beta == 0.0);
  cp->m = g.m;
  cp->j0 = 0;
  cp->j1 = g.n;
  cp->row_exp = rexp;
  cp->col_exp = cexp;
  cp->alpha = g.alpha;
  cp->beta = g.beta;
  cp->c = static_cast<double*>(g.c.ptr);
  cp->rsc = g.c.rs;
  cp->csc = g.c.cs;
}

// One recombination launch over columns [j0, j1) of C on stream Y.
int launch_combine(CombineParams cp, int64_t j0, int64_t j1, int sm_count, cudaStream_t Y) {
  cp.j0 = j0;
  cp.j1 = j1;
  const int64_t bx = ceil_div(cp.m, 512);
  const int64_t by = std::min<int64_t>({j1 - j0, 65535, std::max<int64_t>(1, (int64_t)sm_count * 16 / bx)});
  {
    KernelTimer kt(MOMMS_KERNEL_COMBINE, Y);
    const dim3 grid((unsigned)bx, (unsigned)by);
    switch (cp.levels ? cp.levels : (cp.wide ? -1 : 0)) {
      case -1: combine_kernel<true, 0><<<grid, 256, 0, Y>>>(cp); break;
      case 13: combine_kernel<true, 13><<<grid, 256, 0, Y>>>(cp); break;
      case 14: combine_kernel<true, 14><<<grid, 256, 0, Y>>>(cp); break;
      case 15: combine_kernel<true, 15><<<grid, 256, 0, Y>>>(cp); break;
      case 1: combine_kernel<false, 1><<<grid, 256, 0, Y>>>(cp); break;
      case 2: combine_kernel<false, 2><<<grid, 256, 0, Y>>>(cp); break;
      case 3: combine_kernel<false, 3><<<grid, 256, 0, Y>>>(cp); break;
      case 4: combine_kernel<false, 4><<<grid, 256, 0, Y>>>(cp); break;
      case 5: combine_kernel<false, 5><<<grid, 256, 0, Y>>>(cp); break;
      case 6: combine_kernel<false, 6><<<grid, 256, 0, Y>>>(cp); break;
      case 7: combine_kernel<false, 7><<<grid, 256, 0, Y>>>(cp); break;
      case 8: combine_kernel<false, 8><<<grid, 256, 0, Y>>>(cp); break;
      case 9: combine_kernel<false, 9><<<grid, 256, 0, Y>>>(cp); break;
      case 10: combine_kernel<false, 10><<<grid, 256, 0, Y>>>(cp); break;
      case 11: combine_kernel<false, 11><<<grid, 256, 0, Y>>>(cp); break;
      case 12: combine_kernel<false, 12><<<grid, 256, 0, Y>>>(cp); break;
      default: combine_kernel<false, 0><<<grid, 256, 0, Y>>>(cp); break;
    }
  }
  note_launch();
  const cudaError_t e = launch_status();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "Ozaki launch");
}
}  // namespace

int ozaki_group_count(int ns, int64_t k) {
  Schedule sc;
  return ozaki_schedule(ns, k, &sc) ? sc.ng : sp::MAX_GROUPS;
}

namespace {
constexpr int kMaxChunks = 8;

// Column chunks of one emulated call: n cut at multiples of the tile width.
// Calls whose B / C arrive from host memory take 5 chunks (column_cuts; 4
// equal chunks took 4096^3 e2e from 5.40 to 4.60 ms and 8192^3 from 31.2 to
// 28.3 ms with 7-bit digits; 6 or 8 equal chunks were no better).
// Device-resident calls run unchunked: chunks there
// only moved the next chunk's preparation into the products' tail (8192^3:
// 20.65 vs 20.55 ms, 4096^3: 2.81 vs 2.77 ms), and one launch keeps the
// slice kernel's own timing clean.
// MOMMS_OZAKI_CHUNKS=1..8 fixes the count for A/B measurements; the results
// are the same for every count (each entry's sums do not depend on it).
int column_chunks(int64_t m, int64_t n, int64_t k, bool deferred) {
  (void)m;
  (void)k;
  const char* env = getenv("MOMMS_OZAKI_CHUNKS");
  if (env && *env) {
    const int v = atoi(env);
    if (v >= 1 && v <= kMaxChunks) return (int)std::min<int64_t>(v, ceil_div(n, sp::BN));
  }
  if (deferred) return n >= 2048 ? 5 : (n >= 1024 ? 2 : 1);
  return 1;
}

// Chunk boundaries (multiples of the tile width, the last at n). Five chunks
// of host-staged operands are cut 1/8, 1/4, 1/4, 1/4, 1/8: the first chunk's
// B copy delays the first slice products, and the last chunk's copy-back
// follows them, so both ends are narrow.
void column_cuts(int64_t n, int nch, bool deferred, int64_t* cut) {
  static const int kEighths[6] = {0, 1, 3, 5, 7, 8};
  for (int c = 0; c < nch; ++c) {
    const int64_t x = (deferred && nch == 5) ? n * kEighths[c] / 8 : n * c / nch;
    cut[c] = std::min<int64_t>(n, round_up(x, sp::BN));
  }
  cut[nch] = n;
}
}  // namespace

namespace {

// ---- The guaranteed bound -------------------------------------------------
// Rigorous componentwise bound of an s-slice product relative to |A||B|, from
// the maxima q1 = max (sum|a_i.| 2^-e_i + sum|b_.j| 2^-f_j) / L_ij and
// q2 = max k / L_ij (L_ij <= (|A||B|)_ij 2^-(e_i+f_j)): digit rounding of A and
// B costs 2^(-8s-1) (q1 + 2^(-8s-1) q2), and the diagonals beyond s+1 that the
// triangular scheme drops (pairs of centred digits, |d| <= 2^7) at most
// 2^(-8s-1) (s-1)/2 (256/255) q2.
double guaranteed_bound(int s, double q1, double q2) {
  const double u = ldexp(1.0, -kDigitBits * s - 1);
  return u * (q1 + (0.5 * (s - 1) * (256.0 / 255.0) + u) * q2);
}
double target_or_fp64(double target) { return target > 0.0 ? target : ldexp(1.0, -52); }
// Smallest slice count (at most kOzakiMaxSlices) whose guaranteed bound
// meets the target; *reachable is false if the most slices do not, or if some
// entry is uncovered.
int guaranteed_slices(double target, double q1, double q2, bool uncovered, bool* reachable) {
  const double tgt = target_or_fp64(target);
  int ns = 1;
  while (ns < kOzakiMaxSlices && guaranteed_bound(ns, q1, q2) > tgt) ++ns;
  *reachable = !uncovered && guaranteed_bound(ns, q1, q2) <= tgt;
  return uncovered ? kOzakiMaxSlices : ns;
}

// Scratch of the bound: bf16 magnitude planes of A (m rows) and of B
// transposed (n rows), K-major with row stride kp; the rows' sums of scaled
// magnitudes (units of 2^-40, m then n, contiguous) and the result words
// right after them: out[0], out[1] the maxima (float bits), out[2..3] a
// 64-bit count of covered entries.
struct BoundWork {
  uint16_t* mag_a;
  uint16_t* mag_b;
  unsigned long long* sum_a;
  unsigned long long* sum_b;
  unsigned* out;
  int64_t kp;
};
size_t bound_work_bytes(int64_t m, int64_t n, int64_t k) {
  const int64_t kp = round_up(k, 8);
  return (size_t)round_up(m * kp * 2, 256) + (size_t)round_up(n * kp * 2, 256) + (size_t)(m + n) * 8 + 16;
}
void bound_work_carve(void* base, int64_t m, int64_t n, int64_t k, BoundWork* w) {
  char* p = static_cast<char*>(base);
  w->kp = round_up(k, 8);
  w->mag_a = reinterpret_cast<uint16_t*>(p);
  p += round_up(m * w->kp * 2, 256);
  w->mag_b = reinterpret_cast<uint16_t*>(p);
  p += round_up(n * w->kp * 2, 256);
  w->sum_a = reinterpret_cast<unsigned long long*>(p);
  w->sum_b = w->sum_a + m;
  w->out = reinterpret_cast<unsigned*>(w->sum_b + n);
}

// Magnitude plane and row sums of an R x K view (element (r, p) at
// x[r*sr + p*sp]) under the row exponents, in the run layout of planes.cuh:
// a thread converts runs of 8 elements of one row (one 16-byte store of bf16
// each) and adds their fixed-point terms in a register; the lanes of one
// row (4, or 2^lg) add their terms by shuffles and one of them posts a 64-bit
// atomicAdd. The sums are exact integers, so they do not depend on the order
// of the atomics. With `indicator` the kernel writes the 0/1 plane of nonzero
// elements and no sums.
template <bool R_CONTIG>
__global__ void __launch_bounds__(planes::THREADS)
    magnitude_kernel(const double* __restrict__ x, int64_t sr, int64_t sp, int64_t R, int64_t K, bool vec, int lg,
                     const int* __restrict__ exps, uint16_t* __restrict__ plane, int64_t ldp,
                     unsigned long long* __restrict__ sums, bool indicator) {
  constexpr int RUN = 8;
  const planes::Chunk<R_CONTIG> c(lg);
  // the row loop's trip count is the same for every thread of the block
  // (rows past R only skip their work), so every lane reaches the shuffles
  for (int64_t rb = (int64_t)blockIdx.y * c.rows; rb < R; rb += (int64_t)gridDim.y * c.rows) {
    const int64_t r = rb + c.rl;
    unsigned long long t = 0;
    if (r < R) {
      const int e = exps[r];
      const double* xr = x + r * sr;
      uint16_t* outr = plane + r * ldp;
#pragma unroll 1
      for (int it = 0; it < planes::PITER; ++it) {
        const int64_t p = planes::run_col(blockIdx.x, c, it, RUN);
        if (p >= K) break;
        double v[RUN];
        planes::load_run<R_CONTIG, RUN>(xr, sp, p, K, vec, v);
        uint32_t w[RUN / 2];
#pragma unroll
        for (int q = 0; q < RUN / 2; ++q) {
          uint16_t b0, b1;
          unsigned long long f0, f1;
          magnitude(v[2 * q], e, indicator, &b0, &f0);
          magnitude(v[2 * q + 1], e, indicator, &b1, &f1);
          w[q] = (uint32_t)b0 | ((uint32_t)b1 << 16);
          t += f0 + f1;
        }
        *reinterpret_cast<uint4*>(outr + p) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
    if (indicator) continue;
    // a row's lanes differ in the top lg lane bits (rows contiguous) or in the low lg bits
    if (R_CONTIG) {
      for (int o = 16; o >= (32 >> lg); o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    } else {
      for (int o = c.runs >> 1; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    if (c.ru == 0 && r < R && t) atomicAdd(&sums[r], t);
  }
}

int enqueue_magnitudes(const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K, const int* exps,
                       uint16_t* plane, int64_t kp, unsigned long long* sums, cudaStream_t s, bool indicator = false) {
  if (R == 0) return MOMMS_OK;
  const bool r_contig = (sr == 1 && sp != 1);
  const bool vec = planes::rows_vector_aligned(x, sr, sp);
  if (kp % 8 || (reinterpret_cast<uintptr_t>(plane) & 15))
    return fail(MOMMS_ERR_INVALID_ARG, "Ozaki bound magnitudes: plane rows not 16-byte aligned");
  const int lg = planes::run_lanes_log2(K, 8, r_contig, planes::kRowsContigLg);
  {
    KernelTimer kt(MOMMS_KERNEL_PREP, s);
    if (r_contig)
      magnitude_kernel<true><<<planes::run_grid<true, 8>(R, K, lg), planes::THREADS, 0, s>>>(
          x, sr, sp, R, K, vec, lg, exps, plane, kp, sums, indicator);
    else
      magnitude_kernel<false><<<planes::run_grid<false, 8>(R, K, lg), planes::THREADS, 0, s>>>(
          x, sr, sp, R, K, vec, lg, exps, plane, kp, sums, indicator);
  }
  note_launch();
  const cudaError_t e = launch_status();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "Ozaki bound magnitudes");
}

// The bound kernel (bf16 magnitude product on tcgen05, EPI_BOUND) over all of
// C; the maxima land in w.out[0..1].
int enqueue_bound_kernel(const BoundWork& w, int64_t m, int64_t n, int64_t k, bool count_only, unsigned* status,
                         int sm_count, cudaStream_t s) {
  CUtensorMap tmA, tmB, tmB_half;
  uint64_t dims[3] = {(uint64_t)k, (uint64_t)m, 1};
  uint64_t strides[2] = {(uint64_t)w.kp * 2, (uint64_t)m * w.kp * 2};
  uint32_t box[3] = {64, (uint32_t)sp::BM, 1};
  int rc = encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, w.mag_a, dims, strides, box,
                        CU_TENSOR_MAP_SWIZZLE_128B);
  if (rc) return rc;
  uint64_t dimsb[3] = {(uint64_t)k, (uint64_t)n, 1};
  uint64_t stridesb[2] = {(uint64_t)w.kp * 2, (uint64_t)n * w.kp * 2};
  uint32_t boxb[3] = {64, (uint32_t)sp::BN, 1};
  rc = encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, w.mag_b, dimsb, stridesb, boxb,
                    CU_TENSOR_MAP_SWIZZLE_128B);
  if (rc) return rc;
  uint32_t boxh[3] = {64, (uint32_t)(sp::BN / 2), 1};
  rc = encode_tiled(&tmB_half, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, w.mag_b, dimsb, stridesb, boxh,
                    CU_TENSOR_MAP_SWIZZLE_128B);
  if (rc) return rc;
  sp::Params p;
  memset(&p, 0, sizeof(p));
  p.m = m;
  p.n = n;
  p.kelems = 64;
  p.kblocks = (int)ceil_div(k, 64);
  p.tiles_m = (int)ceil_div(m, sp::BM);
  p.tiles_n = (int)ceil_div(n, sp::BN);
  p.ngroups = 1;
  p.group_begin[0] = 0;
  p.group_begin[1] = 1;
  p.pair_a[0] = 0;
  p.pair_b[0] = 0;
  p.pair_w[0] = 1;
  p.chunk_cap = std::max(1, p.kblocks);  // one FP32 accumulation over all of k
  p.merge_pairs = 0;
  p.msum_a = w.sum_a;
  p.msum_b = w.sum_b;
  // The FP32 sum of non-negative exact bf16 products, accumulated by the
  // tensor core (alignment and truncation at most a few units of 2^-24 per
  // step), is taken to lose at most max(k, 64) 2^-21 of itself.
  const double lbs = 1.0 - (double)std::max<int64_t>(k, 64) * ldexp(1.0, -21);
  p.lb_scale = (float)lbs;
  if ((double)p.lb_scale > lbs) p.lb_scale = nextafterf(p.lb_scale, 0.0f);  // rounded down
  p.kf = (float)k;
  p.bound_out = w.out;
  p.bound_count = reinterpret_cast<unsigned long long*>(w.out + 2);
  p.count_only = count_only ? 1 : 0;
  p.status = status;
  cudaError_t ce;
  {
    KernelTimer kt(MOMMS_KERNEL_BOUND, s);
    int variant = 0;
    ce = sp::launch_slice<2, sp::EPI_BOUND>(tmA, tmB, tmB_half, p, sm_count, s, &variant);
    if (ce == cudaSuccess) ce = launch_status();
  }
  note_launch();
  return ce == cudaSuccess ? MOMMS_OK : cuda_fail(ce, "Ozaki bound launch");
}

// The bound's result, once the bound kernel is enqueued on `s`: the two
// maxima, and whether some entry is uncovered. The kernel counts the entries
// whose lower bound is zero (none, for dense data); if there are any, a
// second pass over 0/1 indicator planes counts the entries with any nonzero
// product term. An entry counted there but without a positive bound has every
// term below FP32's range (relative to 2^(e_i+f_j)): no slice count can vouch
// for it. Entries with no nonzero term are exact (their digits are all zero).
// Synchronises `s`.
struct OperandViews {
  const double* a;
  int64_t a_rs, a_cs;
  const double* b;
  int64_t b_rs, b_cs;
  const int* rexp;
  const int* cexp;
};
int bound_result(const BoundWork& w, const OperandViews& v, int64_t m, int64_t n, int64_t k, DeviceState* ds,
                 cudaStream_t s, float* q1, float* q2, bool* uncovered) {
  unsigned words[4] = {0, 0, 0, 0};
  cudaError_t ce = cudaMemcpyAsync(words, w.out, sizeof(words), cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki bound");
  memcpy(q1, &words[0], 4);
  memcpy(q2, &words[1], 4);
  unsigned long long zeros;
  memcpy(&zeros, &words[2], 8);
  *uncovered = false;
  if (zeros == 0) return MOMMS_OK;
  const unsigned long long covered = (unsigned long long)m * (unsigned long long)n - zeros;
  // indicator pass (sparse operands, or terms beyond FP32's range)
  ce = cudaMemsetAsync(w.out + 2, 0, 8, s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki bound");
  int rc = enqueue_magnitudes(v.a, v.a_rs, v.a_cs, m, k, v.rexp, w.mag_a, w.kp, nullptr, s, true);
  if (!rc) rc = enqueue_magnitudes(v.b, v.b_cs, v.b_rs, n, k, v.cexp, w.mag_b, w.kp, nullptr, s, true);
  if (!rc) rc = enqueue_bound_kernel(w, m, n, k, true, ds->status, ds->sm_count, s);
  if (rc) return rc;
  unsigned long long nonzero = 0;
  ce = cudaMemcpyAsync(&nonzero, w.out + 2, 8, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki bound");
  *uncovered = nonzero > covered;
  return MOMMS_OK;
}

// Events of one emulated call's streams.
struct Events {
  cudaEvent_t fork = nullptr, join = nullptr, join2 = nullptr, bound = nullptr;
  cudaEvent_t mag[kMaxChunks] = {}, prod[kMaxChunks] = {};
  int create(int nch) {
    cudaError_t e = cudaSuccess;
    for (cudaEvent_t* p : {&fork, &join, &join2, &bound})
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(p, cudaEventDisableTiming);
    for (int c = 0; c < nch && e == cudaSuccess; ++c) {
      e = cudaEventCreateWithFlags(&mag[c], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&prod[c], cudaEventDisableTiming);
    }
    return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "Ozaki chunk events");
  }
  void destroy() {
    for (cudaEvent_t* p : {&fork, &join, &join2, &bound})
      if (*p) cudaEventDestroy(*p);
    for (int c = 0; c < kMaxChunks; ++c) {
      if (mag[c]) cudaEventDestroy(mag[c]);
      if (prod[c]) cudaEventDestroy(prod[c]);
    }
  }
};

}  // namespace

int launch_dgemm_ozaki(const DevGemm& g, double target, int slices, int* slices_used, cudaStream_t s) {
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  if (g.k > kMaxK) {
    if (g.pk[0] || g.pk[1])
      return fail(MOMMS_ERR_UNSUPPORTED, "packed operands need k <= %lld (longer k runs in re-scaled slabs)",
                  (long long)kMaxK);
    // k slabs of at most kMaxK (the int32 digit sums' range), later slabs
    // accumulating into C with beta = 1 like the reference's PartK
    // (src/composables/part.rs:96-110); each slab meets the target on its own
    const int64_t nslab = ceil_div(g.k, kMaxK), kb = round_up(ceil_div(g.k, nslab), 64);
    bool unreachable = false;
    // deferred B / C arrive whole before the first slab
    for (int w = 1; w <= 2 && g.staging; ++w)
      if (g.staging->deferred[w]) {
        cudaEvent_t ev = nullptr;
        const int rc = copy_columns(g, w, 0, g.n, &ev);
        if (rc) return rc;
        g.staging->deferred[w] = false;
        g.staging->ready[w] = ev;
      }
    for (int64_t p0 = 0; p0 < g.k; p0 += kb) {
      DevGemm gs = g;
      gs.k = std::min(kb, g.k - p0);
      gs.a.ptr = static_cast<double*>(g.a.ptr) + p0 * g.a.cs;
      gs.b.ptr = static_cast<double*>(g.b.ptr) + p0 * g.b.rs;
      if (p0 > 0) {
        gs.beta = 1.0;
        gs.staging = nullptr;  // the first slab waited for the operands
      } else if (g.staging) {
        gs.staging->writeback = nullptr;  // C goes back after the last slab
      }
      int rc = launch_dgemm_ozaki(gs, target, slices, slices_used, s);
      if (rc == MOMMS_ERR_TARGET_UNREACHABLE) unreachable = true;
      else if (rc) return rc;
    }
    return unreachable ? MOMMS_ERR_TARGET_UNREACHABLE : MOMMS_OK;
  }
  const int bits = kDigitBits;
  const int64_t m = g.m, n = g.n, k = g.k;
  cudaError_t ce;

  // Packed operands bring their exponents and digit planes, and fix the slice
  // count (no sampled choice, no host round trip).
  const PackedOperand* PA = g.pk[0];
  const PackedOperand* PB = g.pk[1];
  int ns_fixed = 0;
  if (PA) ns_fixed = PA->np;
  if (PB) {
    if (ns_fixed && PB->np != ns_fixed)
      return fail(MOMMS_ERR_INVALID_ARG, "packed A has %d slices, packed B %d", ns_fixed, PB->np);
    ns_fixed = PB->np;
  }
  if (ns_fixed && slices > 0 && slices != ns_fixed)
    return fail(MOMMS_ERR_INVALID_ARG, "desc asks for %d slices, the packed operand holds %d", slices, ns_fixed);

  // Column chunks (column_chunks): chunk c runs on s (even c) or the
  // device's second compute stream (odd c), so that chunk c+1's B
  // preparation and chunk c's recombination fill the tail of chunk c's slice
  // products, and deferred B / C columns arrive a chunk ahead of their use.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  Staging* stg = g.staging;
  const bool defer_b = stg && stg->deferred[1], defer_c = stg && stg->deferred[2];
  const int nch = (cap == cudaStreamCaptureStatusNone && ds->aux) ? column_chunks(m, n, k, defer_b || defer_c) : 1;
  int64_t cut[kMaxChunks + 1];
  column_cuts(n, nch, defer_b || defer_c, cut);
  const bool choose = ns_fixed == 0 && slices <= 0;

  // Deferred copies in the order they are read: B's sampled columns (the
  // slice-count choice needs only those), then B's chunks, each C chunk one
  // behind its B chunk.
  cudaEvent_t ev_sample = nullptr, ev_b[kMaxChunks] = {}, ev_c[kMaxChunks] = {};
  int rc = MOMMS_OK;
  if (defer_b && choose) {
    int64_t js[kSamples];
    for (int q = 0; q < kSamples; ++q) {
      int64_t i0;
      sample_position(q % kSampleRowBlocks, q / kSampleRowBlocks, m, n, &i0, &js[q]);
    }
    std::sort(js, js + kSamples);
    for (int q = 0; q < kSamples && !rc;) {
      int r = q + 1;
      while (r < kSamples && js[r] <= js[r - 1] + 1) ++r;  // a run of adjacent or repeated columns
      rc = copy_columns(g, 1, js[q], js[r - 1] + 1, r == kSamples ? &ev_sample : nullptr);
      q = r;
    }
  }
  for (int c = 0; c < nch && !rc; ++c) {
    if (defer_b) rc = copy_columns(g, 1, cut[c], cut[c + 1], &ev_b[c]);
    if (!rc && defer_c && c > 0) rc = copy_columns(g, 2, cut[c - 1], cut[c], &ev_c[c - 1]);
  }
  if (!rc && defer_c) rc = copy_columns(g, 2, cut[nch - 1], cut[nch], &ev_c[nch - 1]);
  if (rc) return rc;

  // exponents of the unpacked operands: [m + n] u64 maxima, [m + n] int exponents
  void* ebuf = nullptr;
  if ((ce = scratch_alloc(&ebuf, (size_t)(m + n) * (sizeof(unsigned long long) + sizeof(int)), s)) != cudaSuccess)
    return cuda_fail(ce, "Ozaki exponents");
  ScratchGuard free_ebuf(ebuf, s);
  unsigned long long* maxbits = static_cast<unsigned long long*>(ebuf);
  int* exps = reinterpret_cast<int*>(maxbits + (m + n));
  const double* A = static_cast<const double*>(g.a.ptr);
  const double* B = static_cast<const double*>(g.b.ptr);
  if ((ce = wait_operand(g, 0, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
  if (!PA) rc = ozaki_operand_exponents(A, g.a.rs, g.a.cs, m, k, maxbits, exps, s);
  if (rc) return rc;
  const int* rexp = PA ? PA->exps : exps;
  int* cexp_w = exps + m;  // B's column exponents, written per chunk
  const int* cexp = PB ? PB->exps : cexp_w;

  int ns = ns_fixed ? ns_fixed : slices;
  // Automatic count, guaranteed for every entry by the bound kernel (the
  // bf16 magnitude product, about 1/28 of the slice products' tensor work):
  //  * operands on the device (B not deferred): the bound runs first and the
  //    count comes from it (one synchronisation, as the choice always had);
  //  * B arriving from host memory by column chunks: a sampled estimate
  //    starts the work on A and the first chunks early, the bound follows once
  //    all of B is in, and the recombinations (the only kernels writing C)
  //    wait for its verdict; a count that misses the target is redone with the
  //    bound's count while C still holds its input.
  const bool automatic = ns <= 0;
  const bool verify = automatic && defer_b;
  bool b_exps_ready = false;
  int verdict = MOMMS_OK;
  BoundWork bw{};
  void* bw_mem = nullptr;
  if (automatic) {
    if ((ce = scratch_alloc(&bw_mem, bound_work_bytes(m, n, k), s)) != cudaSuccess)
      return cuda_fail(ce, "Ozaki bound scratch");
    bound_work_carve(bw_mem, m, n, k, &bw);
    // sums and result words start at zero (they are contiguous); A's
    // magnitudes on s after A's exponents
    ce = cudaMemsetAsync(bw.sum_a, 0, (size_t)(m + n) * sizeof(unsigned long long) + 4 * sizeof(unsigned), s);
    rc = ce == cudaSuccess ? enqueue_magnitudes(A, g.a.rs, g.a.cs, m, k, rexp, bw.mag_a, bw.kp, bw.sum_a, s)
                           : cuda_fail(ce, "Ozaki bound scratch");
    if (rc) {
      cudaFreeAsync(bw_mem, s);
      return rc;
    }
  }
  ScratchGuard free_bw(bw_mem, s);
  if (automatic && !verify) {
    // all of B's exponents and magnitudes, the bound, the count
    if ((ce = wait_operand(g, 1, s)) != cudaSuccess) return cuda_fail(ce, "operand staging");
    rc = ozaki_operand_exponents(B, g.b.cs, g.b.rs, n, k, maxbits + m, cexp_w, s);
    if (!rc) rc = enqueue_magnitudes(B, g.b.cs, g.b.rs, n, k, cexp_w, bw.mag_b, bw.kp, bw.sum_b, s);
    if (!rc) rc = enqueue_bound_kernel(bw, m, n, k, false, ds->status, ds->sm_count, s);
    float q1f = 0.0f, q2f = 0.0f;
    bool uncovered = false;
    if (!rc)
      rc = bound_result(bw, OperandViews{A, g.a.rs, g.a.cs, B, g.b.rs, g.b.cs, rexp, cexp_w}, m, n, k, ds, s, &q1f,
                        &q2f, &uncovered);
    if (rc) return rc;
    bool reachable = false;
    ns = guaranteed_slices(target, q1f, q2f, uncovered, &reachable);
    call_info().bound_rel_err = uncovered ? HUGE_VAL : guaranteed_bound(ns, q1f, q2f);
    if (!reachable) verdict = MOMMS_ERR_TARGET_UNREACHABLE;
    b_exps_ready = true;
  } else if (automatic) {
    // B at the sampled columns, and their exponents
    if ((ce = cudaStreamWaitEvent(s, ev_sample, 0)) != cudaSuccess) return cuda_fail(ce, "operand staging");
    {
      KernelTimer kt(MOMMS_KERNEL_PREP, s);
      sample_col_exps_kernel<<<kSamples, 256, 0, s>>>(B, g.b.rs, g.b.cs, m, n, k, cexp_w);
    }
    note_launch();
    rc = choose_slices(g, rexp, cexp_w, target, bits, s, &ns, nullptr);
    if (rc) return rc;
  }
  if (slices_used) *slices_used = ns;

  const int64_t kp = round_up(k, 8);  // 16-byte rows of fp16
  const size_t a_plane = (size_t)m * kp, b_plane = (size_t)n * kp;
  __half* planes_buf = nullptr;
  const size_t own = (PA ? 0 : (size_t)ns * a_plane) + (PB ? 0 : (size_t)ns * b_plane);
  if (own && (ce = scratch_alloc(&planes_buf, own * sizeof(__half), s)) != cudaSuccess)
    return cuda_fail(ce, "Ozaki slice planes");
  ScratchGuard free_planes(planes_buf, s);
  const __half* pa = PA ? static_cast<const __half*>(PA->planes) : planes_buf;
  const __half* pb = PB ? static_cast<const __half*>(PB->planes) : planes_buf + (PA ? 0 : (size_t)ns * a_plane);
  if (!PA) ozaki_operand_planes(ns, A, g.a.rs, g.a.cs, m, k, const_cast<__half*>(pa), kp, rexp, s);

  if (k > kMaxK) return fail(MOMMS_ERR_UNSUPPORTED, "Ozaki emulation supports k <= %lld per launch", (long long)kMaxK);
  CUtensorMap tmA;
  {
    uint64_t dims[3] = {(uint64_t)k, (uint64_t)m, (uint64_t)ns};
    uint64_t strides[2] = {(uint64_t)kp * 2, (uint64_t)a_plane * 2};
    uint32_t box[3] = {64, (uint32_t)sp::BM, 1};  // 128-byte k-blocks
    rc = encode_tiled(&tmA, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, pa, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) return rc;
  }

  sp::Params p;
  Schedule sch;
  if (!slice_params(ns, m, k, &p, &sch)) return fail(MOMMS_ERR_UNSUPPORTED, "Ozaki schedule needs too many groups");
  const int np = sch.np, ng = sch.ng;
  call_info().slices = ns;
  call_info().pairs = np;
  call_info().groups = ng;

  int* sbuf = nullptr;
  // group planes tile-blocked (sp::Params::sbuf): m and n padded to whole
  // 128 x 256 tiles, each tile one contiguous block
  const int64_t mpad = round_up(m, (int64_t)sp::BM);
  const size_t plane = (size_t)mpad * (size_t)round_up(n, (int64_t)sp::BN);
  if ((ce = scratch_alloc(&sbuf, (size_t)ng * plane * sizeof(int), s)) != cudaSuccess)
    return cuda_fail(ce, "Ozaki group sums");
  ScratchGuard free_sbuf(sbuf, s);
  p.plane = (int64_t)plane;
  p.status = ds->status;
  CombineParams cp;
  combine_params(g, ns, sch, sbuf, (int64_t)plane, mpad, rexp, cexp, &cp);

  // The second stream starts after everything above (scratch, A, the
  // choice), and so does the verify stream V, which runs the bound kernel
  // and, under verification, the recombinations.
  cudaStream_t V = verify ? ds->aux2 : nullptr;
  Events ev;
  if (nch > 1 || verify) {
    rc = ev.create(nch);
    if (!rc) {
      ce = cudaEventRecord(ev.fork, s);
      if (ce == cudaSuccess && nch > 1) ce = cudaStreamWaitEvent(ds->aux, ev.fork, 0);
      if (ce == cudaSuccess && verify) ce = cudaStreamWaitEvent(V, ev.fork, 0);
      if (ce != cudaSuccess) rc = cuda_fail(ce, "Ozaki chunk streams");
    }
  }
  // Recombination of chunk c (columns j0..j1 of C) on stream Y: with C staged
  // from host memory and one chunk, in column ranges each copied back while
  // the next is computed.
  auto combine_chunk = [&](int c, cudaStream_t Y) -> int {
    const int64_t j0 = cut[c], j1 = cut[c + 1], w = j1 - j0;
    cudaError_t e = defer_c ? cudaStreamWaitEvent(Y, ev_c[c], 0) : wait_operand(g, 2, Y);
    if (e != cudaSuccess) return cuda_fail(e, "operand staging");
    const int64_t nsub = (nch == 1 && stg && stg->writeback) ? std::min<int64_t>(4, w) : 1;
    for (int64_t q = 0; q < nsub; ++q) {
      const int64_t c0 = j0 + w * q / nsub, c1 = j0 + w * (q + 1) / nsub;
      int r2 = launch_combine(cp, c0, c1, ds->sm_count, Y);
      if (!r2) r2 = columns_done(g, c0, c1, Y);
      if (r2) return r2;
    }
    return MOMMS_OK;
  };
  for (int c = 0; c < nch && !rc; ++c) {
    const int64_t j0 = cut[c], j1 = cut[c + 1], w = j1 - j0;
    if (w <= 0) continue;
    cudaStream_t X = (c & 1) ? ds->aux : s;
    // B's columns j0..j1: exponents and digit planes
    ce = defer_b ? cudaStreamWaitEvent(X, ev_b[c], 0) : wait_operand(g, 1, X);
    if (ce != cudaSuccess) {
      rc = cuda_fail(ce, "operand staging");
      break;
    }
    const double* Bc = B + j0 * g.b.cs;
    if (!PB) {
      if (!b_exps_ready) rc = ozaki_operand_exponents(Bc, g.b.cs, g.b.rs, w, k, maxbits + m + j0, cexp_w + j0, X);
      if (rc) break;
      KernelTimer kt(MOMMS_KERNEL_PREP, X);
      ozaki_planes(ns, Bc, g.b.cs, g.b.rs, w, k, const_cast<__half*>(pb) + j0 * kp, kp, (int64_t)b_plane,
                   cexp_w + j0, X);
      note_launch();
    }
    if (verify) {
      // B's magnitudes for the bound (verify implies B is not packed)
      rc = enqueue_magnitudes(Bc, g.b.cs, g.b.rs, w, k, cexp_w + j0, bw.mag_b + j0 * bw.kp, bw.kp, bw.sum_b + j0, X);
      if (rc) break;
      if ((ce = cudaEventRecord(ev.mag[c], X)) != cudaSuccess || (ce = cudaStreamWaitEvent(V, ev.mag[c], 0)) != cudaSuccess) {
        rc = cuda_fail(ce, "Ozaki bound events");
        break;
      }
    }
    CUtensorMap tmB, tmB_half;
    {
      const __half* pbc = pb + j0 * kp;
      uint64_t dimsb[3] = {(uint64_t)k, (uint64_t)w, (uint64_t)ns};
      uint64_t stridesb[2] = {(uint64_t)kp * 2, (uint64_t)b_plane * 2};
      uint32_t boxb[3] = {64, (uint32_t)sp::BN, 1};
      rc = encode_tiled(&tmB, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, pbc, dimsb, stridesb, boxb,
                        CU_TENSOR_MAP_SWIZZLE_128B);
      if (rc) break;
      uint32_t boxh[3] = {64, (uint32_t)(sp::BN / 2), 1};  // one CTA's half of the B tile for the pair kernel
      rc = encode_tiled(&tmB_half, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, pbc, dimsb, stridesb, boxh,
                        CU_TENSOR_MAP_SWIZZLE_128B);
      if (rc) break;
    }
    p.n = w;
    p.tiles_n = (int)ceil_div(w, sp::BN);
    p.sbuf = sbuf + j0 * mpad;  // j0 is a multiple of the tile width: the chunk's tile blocks start here
    {
      KernelTimer kt(MOMMS_KERNEL_SLICE_OZAKI, X);
      int variant = 0;
      ce = sp::launch_slice<0, sp::EPI_OZAKI>(tmA, tmB, tmB_half, p, ds->sm_count, X, &variant);
      if (ce == cudaSuccess) ce = launch_status();
      if (ce != cudaSuccess) {
        rc = cuda_fail(ce, "Ozaki slice launch");
        break;
      }
      call_info().slice_variant = variant;
    }
    note_launch();
    if (verify) {
      // the recombination waits for the bound's verdict (below)
      if ((ce = cudaEventRecord(ev.prod[c], X)) != cudaSuccess) rc = cuda_fail(ce, "Ozaki chunk streams");
    } else {
      rc = combine_chunk(c, X);
    }
  }

  // Verification: the bound kernel over all of C on V, once A's and every B
  // chunk's magnitudes are in; the host reads the two maxima. Nothing has
  // written C yet, so a count that misses the target is simply redone.
  int redo = 0;
  float q1f = 0.0f, q2f = 0.0f;
  bool uncovered = false;
  if (verify && !rc) {
    rc = enqueue_bound_kernel(bw, m, n, k, false, ds->status, ds->sm_count, V);
    if (!rc)
      rc = bound_result(bw, OperandViews{A, g.a.rs, g.a.cs, B, g.b.rs, g.b.cs, rexp, cexp_w}, m, n, k, ds, V, &q1f,
                        &q2f, &uncovered);
    if (!rc) {
      bool reachable = false;
      const int need = guaranteed_slices(target, q1f, q2f, uncovered, &reachable);
      if (need > ns) {
        redo = need;  // more slices: redo with that count (C untouched)
      } else {
        call_info().bound_rel_err = uncovered ? HUGE_VAL : guaranteed_bound(ns, q1f, q2f);
        if (!reachable) verdict = MOMMS_ERR_TARGET_UNREACHABLE;
      }
    }
    for (int c = 0; c < nch && !rc && !redo; ++c) {
      if ((ce = cudaStreamWaitEvent(V, ev.prod[c], 0)) != cudaSuccess) rc = cuda_fail(ce, "Ozaki chunk streams");
      else rc = combine_chunk(c, V);
    }
  }
  // s waits for the other streams' work (also after an error: the scratch
  // the guards free may still be in use there)
  if (nch > 1 || verify) {
    cudaError_t e2 = cudaSuccess;
    if (nch > 1) {
      e2 = cudaEventRecord(ev.join, ds->aux);
      if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, ev.join, 0);
    }
    if (e2 == cudaSuccess && verify) {
      e2 = cudaEventRecord(ev.join2, V);
      if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, ev.join2, 0);
    }
    if (!rc && e2 != cudaSuccess) rc = cuda_fail(e2, "Ozaki chunk streams");
  }
  ev.destroy();
  if (rc) return rc;
  if (redo) {
    // Everything of this attempt is in flight or done on s; the operands are
    // all on the device by now (every deferred copy was issued and s waits
    // for it), so the repeat reads them in place, and C still holds its
    // input values. The count comes from the bound: no sample, no second
    // verification.
    if (stg) {
      // this attempt issued every deferred copy: s waits for C's (B's were
      // waited for by the chunk streams s has joined), and the repeat finds
      // both operands in place
      for (int c = 0; c < nch && defer_c; ++c)
        if (ev_c[c] && (ce = cudaStreamWaitEvent(s, ev_c[c], 0)) != cudaSuccess) return cuda_fail(ce, "operand staging");
      stg->deferred[1] = stg->deferred[2] = false;
      stg->ready[1] = stg->ready[2] = nullptr;
    }
    const int use = std::min(redo, kOzakiMaxSlices);
    rc = launch_dgemm_ozaki(g, target, use, slices_used, s);
    if (rc) return rc;
    const double b = uncovered ? HUGE_VAL : guaranteed_bound(use, q1f, q2f);
    call_info().bound_rel_err = b;
    return b > target_or_fp64(target) ? MOMMS_ERR_TARGET_UNREACHABLE : MOMMS_OK;
  }
  return verdict;  // the guards return the scratch to the pool, in order on s after the joins
}

// The slice count of a plan's emulated problem, chosen once at plan creation
// from the operands' current contents: the smallest count whose guaranteed
// bound meets the target for every entry (exponents, magnitude planes and
// the bound kernel, then one synchronisation). k beyond one launch's limit
// is bounded slab by slab, as the launches compute it.
int ozaki_choose_slices(const momms_gemm_desc& d, int* slices, cudaStream_t s) {
  // a packed operand fixes the count
  const PackedOperand* pa = packed_of(d.a);
  const PackedOperand* pb = packed_of(d.b);
  if (pa || pb) {
    *slices = (pa ? pa : pb)->np;
    return MOMMS_OK;
  }
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  const int64_t m = d.m, n = d.n;
  const int64_t nslab = ceil_div(d.k, kMaxK), kb = round_up(ceil_div(d.k, nslab), 64);
  const int64_t kmax = std::min(d.k, kb);
  void* ebuf = nullptr;
  cudaError_t ce = scratch_alloc(&ebuf, (size_t)(m + n) * (sizeof(unsigned long long) + sizeof(int)), s);
  if (ce != cudaSuccess) return cuda_fail(ce, "Ozaki exponents");
  ScratchGuard free_ebuf(ebuf, s);
  void* bw_mem = nullptr;
  if ((ce = scratch_alloc(&bw_mem, bound_work_bytes(m, n, kmax), s)) != cudaSuccess)
    return cuda_fail(ce, "Ozaki bound scratch");
  ScratchGuard free_bw(bw_mem, s);
  BoundWork bw{};
  unsigned long long* maxbits = static_cast<unsigned long long*>(ebuf);
  int* exps = reinterpret_cast<int*>(maxbits + (m + n));
  int need = 1, rc = MOMMS_OK;
  bool reachable_all = true;
  for (int64_t p0 = 0; p0 < d.k && !rc; p0 += kb) {
    DevGemm g;
    g.m = m;
    g.n = n;
    g.k = std::min(kb, d.k - p0);
    g.a = DevMat{static_cast<double*>(d.a.ptr) + p0 * d.a.cs, d.a.rs, d.a.cs};
    g.b = DevMat{static_cast<double*>(d.b.ptr) + p0 * d.b.rs, d.b.rs, d.b.cs};
    bound_work_carve(bw_mem, m, n, g.k, &bw);
    rc = compute_exponents(g, maxbits, exps, s);
    if (!rc) {
      ce = cudaMemsetAsync(bw.sum_a, 0, (size_t)(m + n) * sizeof(unsigned long long) + 4 * sizeof(unsigned), s);
      if (ce != cudaSuccess) rc = cuda_fail(ce, "Ozaki bound scratch");
    }
    const double* Ap = static_cast<const double*>(g.a.ptr);
    const double* Bp = static_cast<const double*>(g.b.ptr);
    if (!rc) rc = enqueue_magnitudes(Ap, g.a.rs, g.a.cs, m, g.k, exps, bw.mag_a, bw.kp, bw.sum_a, s);
    if (!rc) rc = enqueue_magnitudes(Bp, g.b.cs, g.b.rs, n, g.k, exps + m, bw.mag_b, bw.kp, bw.sum_b, s);
    if (!rc) rc = enqueue_bound_kernel(bw, m, n, g.k, false, ds->status, ds->sm_count, s);
    float q1 = 0.0f, q2 = 0.0f;
    bool uncovered = false;
    if (!rc)
      rc = bound_result(bw, OperandViews{Ap, g.a.rs, g.a.cs, Bp, g.b.rs, g.b.cs, exps, exps + m}, m, n, g.k, ds, s,
                        &q1, &q2, &uncovered);
    if (!rc) {
      bool reachable = false;
      need = std::max(need, guaranteed_slices(d.target_rel_err, q1, q2, uncovered, &reachable));
      reachable_all = reachable_all && reachable;
    }
  }
  if (rc) return rc;
  *slices = need;
  if (!reachable_all)
    return fail(MOMMS_ERR_TARGET_UNREACHABLE,
                "Ozaki: the requested error %.3g cannot be guaranteed for every entry with 15 slices (pass a fixed "
                "slice count to run anyway)",
                target_or_fp64(d.target_rel_err));
  return MOMMS_OK;
}

}  // namespace momms

// ---------------------------------------------------------------------------
// Emulated problems of a plan in one slice launch (OzakiBatch).
// ---------------------------------------------------------------------------
namespace momms {

struct OzakiBatch {
  struct Prob {
    DevGemm g;
    int ns = 0;
    void* mem = nullptr;  // maxbits [m+n] u64, exps [m+n] int, planes, group sums
    unsigned long long* maxbits = nullptr;
    int* exps = nullptr;
    __half* planes = nullptr;
    int* sbuf = nullptr;
    int64_t kp = 0;
    size_t a_plane = 0, b_plane = 0;
    CombineParams cp;
  };
  std::vector<Prob> probs;
  sp::Params* d_params = nullptr;  // device problem table
  CUtensorMap* d_maps = nullptr;   // [2 * count], A and B half-tile maps
  int64_t units = 0;
  bool async = false;
  cudaStream_t stream = nullptr;
};

bool sp_pairs_available(int* clusters) {
  return sp::slice_variant<0, sp::EPI_OZAKI>(clusters) == sp::SLICE_PAIR && *clusters > 0;
}

bool ozaki_batchable(const DevGemm& g, int slices) {
  return slices > 0 && slices <= kOzakiMaxSlices && !g.pk[0] && !g.pk[1] && g.k <= kMaxK && g.m > 0 && g.n > 0 &&
         g.k > 0;
}

void ozaki_batch_destroy(OzakiBatch* b) {
  if (!b) return;
  auto release = [&](void* p) {
    if (!p) return;
    if (b->async) cudaFreeAsync(p, b->stream);
    else cudaFree(p);
  };
  for (auto& pr : b->probs) release(pr.mem);
  release(b->d_params);
  release(b->d_maps);
  delete b;
}

int ozaki_batch_create(const DevGemm* gs, const int* slices, int count, cudaStream_t s, bool async, OzakiBatch** out) {
  *out = nullptr;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  OzakiBatch* b = new OzakiBatch();
  b->async = async;
  b->stream = s;
  auto alloc = [&](void** p, size_t bytes) {
    const cudaError_t e = async ? scratch_alloc_raw(p, bytes, s) : device_malloc(p, bytes);
    return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "Ozaki batch allocation");
  };
  std::vector<sp::Params> params((size_t)count);
  std::vector<CUtensorMap> maps((size_t)count * 2);
  // problems ordered by falling cost (pairs x k-blocks x pair tiles), so the
  // kernel hands out the largest units first
  std::vector<int> order((size_t)count);
  std::vector<double> cost((size_t)count);
  for (int i = 0; i < count; ++i) {
    order[(size_t)i] = i;
    const DevGemm& g = gs[i];
    cost[(size_t)i] = (double)ceil_div(g.m, 2 * sp::BM) * ceil_div(g.n, sp::BN) * ceil_div(g.k, 64) * slices[i] *
                      (slices[i] + 1);
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[(size_t)x] > cost[(size_t)y]; });
  int rc = MOMMS_OK;
  b->probs.resize((size_t)count);
  for (int oi = 0; oi < count && !rc; ++oi) {
    const int i = order[(size_t)oi];
    OzakiBatch::Prob& P = b->probs[(size_t)oi];
    P.g = gs[i];
    P.ns = slices[i];
    const int64_t m = P.g.m, n = P.g.n, k = P.g.k;
    sp::Params& prm = params[(size_t)oi];
    Schedule sch;
    if (!slice_params(P.ns, m, k, &prm, &sch)) {
      rc = fail(MOMMS_ERR_UNSUPPORTED, "Ozaki schedule needs too many groups");
      break;
    }
    P.kp = round_up(k, 8);
    P.a_plane = (size_t)m * P.kp;
    P.b_plane = (size_t)n * P.kp;
    const int64_t mpad = round_up(m, (int64_t)sp::BM);
    const size_t plane = (size_t)mpad * (size_t)round_up(n, (int64_t)sp::BN);
    const size_t eb = (size_t)round_up((m + n) * 12, 256);
    const size_t pb = (size_t)round_up((int64_t)(P.ns * (P.a_plane + P.b_plane) * 2), 256);
    rc = alloc(&P.mem, eb + pb + (size_t)sch.ng * plane * 4);
    if (rc) break;
    char* base = static_cast<char*>(P.mem);
    P.maxbits = reinterpret_cast<unsigned long long*>(base);
    P.exps = reinterpret_cast<int*>(P.maxbits + (m + n));
    P.planes = reinterpret_cast<__half*>(base + eb);
    P.sbuf = reinterpret_cast<int*>(base + eb + pb);
    prm.n = n;
    prm.tiles_n = (int)ceil_div(n, sp::BN);
    prm.sbuf = P.sbuf;
    prm.plane = (int64_t)plane;
    prm.gchunk = prm.ngroups;  // a batch fills the GPU without splitting a tile's groups
    prm.status = ds->status;
    if (!sp::plan_chunks(prm)) {
      rc = fail(MOMMS_ERR_UNSUPPORTED, "Ozaki chunk plan");
      break;
    }
    prm.unit_begin = b->units;
    b->units += (int64_t)((prm.tiles_m + 1) / 2) * prm.tiles_n;
    combine_params(P.g, P.ns, sch, P.sbuf, (int64_t)plane, mpad, P.exps, P.exps + m, &P.cp);
    // A [ns][m][kp] and B [ns][n][kp], 128-byte k-blocks, each CTA of a pair
    // staging half of the 256-row B tile
    uint64_t dims[3] = {(uint64_t)k, (uint64_t)m, (uint64_t)P.ns};
    uint64_t strides[2] = {(uint64_t)P.kp * 2, (uint64_t)P.a_plane * 2};
    uint32_t box[3] = {64, (uint32_t)sp::BM, 1};
    rc = encode_tiled(&maps[2 * (size_t)oi], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, P.planes, dims, strides, box,
                      CU_TENSOR_MAP_SWIZZLE_128B);
    if (rc) break;
    uint64_t dimsb[3] = {(uint64_t)k, (uint64_t)n, (uint64_t)P.ns};
    uint64_t stridesb[2] = {(uint64_t)P.kp * 2, (uint64_t)P.b_plane * 2};
    uint32_t boxh[3] = {64, (uint32_t)(sp::BN / 2), 1};
    rc = encode_tiled(&maps[2 * (size_t)oi + 1], CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, P.planes + P.ns * P.a_plane,
                      dimsb, stridesb, boxh, CU_TENSOR_MAP_SWIZZLE_128B);
  }
  if (!rc) rc = alloc(reinterpret_cast<void**>(&b->d_params), params.size() * sizeof(sp::Params));
  if (!rc) rc = alloc(reinterpret_cast<void**>(&b->d_maps), maps.size() * sizeof(CUtensorMap));
  if (!rc) {
    // synchronous uploads: the host tables need not outlive this call
    cudaError_t e = cudaMemcpyAsync(b->d_params, params.data(), params.size() * sizeof(sp::Params),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = cuda_fail(e, "Ozaki batch tables");
  }
  if (rc) {
    ozaki_batch_destroy(b);
    return rc;
  }
  *out = b;
  return MOMMS_OK;
}

int ozaki_batch_launch(OzakiBatch* b, cudaStream_t s, int max_sms) {
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  if (b->probs.empty()) return MOMMS_OK;
  // each problem's exponents and digit planes
  for (auto& P : b->probs) {
    const DevGemm& g = P.g;
    const double* A = static_cast<const double*>(g.a.ptr);
    const double* B = static_cast<const double*>(g.b.ptr);
    int rc = ozaki_operand_exponents(A, g.a.rs, g.a.cs, g.m, g.k, P.maxbits, P.exps, s);
    if (!rc) rc = ozaki_operand_exponents(B, g.b.cs, g.b.rs, g.n, g.k, P.maxbits + g.m, P.exps + g.m, s);
    if (rc) return rc;
    ozaki_operand_planes(P.ns, A, g.a.rs, g.a.cs, g.m, g.k, P.planes, P.kp, P.exps, s);
    ozaki_operand_planes(P.ns, B, g.b.cs, g.b.rs, g.n, g.k, P.planes + P.ns * P.a_plane, P.kp, P.exps + g.m, s);
  }
  // one persistent slice launch over every problem's tiles
  int clusters = 0;
  if (sp::slice_variant<0, sp::EPI_OZAKI>(&clusters) != sp::SLICE_PAIR || clusters <= 0)
    return fail(MOMMS_ERR_UNSUPPORTED, "grouped emulated launches need CTA pairs on this device");
  if (max_sms > 0) clusters = std::max(1, std::min(clusters, max_sms / 2));
  sp::GroupTable gt{b->d_params, b->d_maps, (int)b->probs.size(), b->units};
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = sp::cluster2_config(sp::P_SMEM_BYTES, attr);
  cfg.gridDim = dim3((unsigned)(2 * std::min<int64_t>(b->units, clusters)));
  cfg.stream = s;
  cudaError_t e;
  {
    KernelTimer kt(MOMMS_KERNEL_SLICE_OZAKI, s);
    const CUtensorMap unused{};
    e = cudaLaunchKernelEx(&cfg, sp::slice_gemm_pair_kernel<0, sp::EPI_OZAKI, true>, unused, unused, sp::Params{},
                           gt);
    if (e == cudaSuccess) e = launch_status();
  }
  note_launch();
  if (e != cudaSuccess) return cuda_fail(e, "grouped Ozaki slice launch");
  for (auto& P : b->probs) {
    const int rc = launch_combine(P.cp, 0, P.g.n, ds->sm_count, s);
    if (rc) return rc;
  }
  return MOMMS_OK;
}

}  // namespace momms
