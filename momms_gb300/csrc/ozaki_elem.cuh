// Element-wise arithmetic of the Ozaki operand passes, on the bit pattern of
// each double (GB300's FP64 pipe is about 1 TFLOP/s, so FP64 arithmetic per
// element would dominate the passes): the magnitude order of |v|, a row's
// exponent from its largest magnitude, an element's offset digits, and its
// terms of the bound (a bf16 magnitude rounded toward zero and an upward
// fixed-point term of the row sum).
//
// Host-callable (the device branches use the CUDA intrinsics, the host ones
// portable equivalents), so that tests check every function against exact
// rational arithmetic on the CPU.
#pragma once
#include <stdint.h>
#include <string.h>

#include "exact_round.cuh"

namespace momms {
namespace elem {

constexpr int kDigitBits = 8;  // bits per Ozaki digit

// |v| as an unsigned bit pattern: for non-negative doubles the unsigned order
// of the patterns is the order of the values; infinities and NaNs sort above
// every finite value.
__host__ __device__ __forceinline__ unsigned long long abs_bits(double v) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
#else
  unsigned long long b;
  memcpy(&b, &v, sizeof b);
  return b & 0x7fffffffffffffffull;
#endif
}

// Exponent e of a row whose largest |v| has bit pattern b: |v| < 2^e (the
// frexp exponent of the maximum); 0 for an all-zero row; INT32_MAX for a row
// holding a NaN or an infinity.
__host__ __device__ __forceinline__ int exponent_of_max(unsigned long long b) {
  if (b >= 0x7ff0000000000000ull) return INT32_MAX;
  if (b == 0) return 0;
  if ((b >> 52) != 0) return (int)(b >> 52) - 1022;  // [2^(be-1023), 2^(be-1022))
  return (63 - clz64(b)) - 1073;                      // subnormal
}

// Signed digits of v * 2^-e at kDigitBits bits each, nearest rounding at the
// last digit: X = round(|v| * 2^(bits*NS - e)) as an integer, written as
//   X = sum_{pos < NS-1} d_pos 2^(bits*pos) + top 2^(bits*(NS-1))
// with centred lower digits d_pos in [-2^(bits-1), 2^(bits-1)) and the top
// digit in [0, 2^bits]. That representation is unique, and all its digits come
// at once from Y = X + H, H = 2^(bits-1) * sum_{pos < NS-1} 2^(bits*pos):
// Y's plain base-2^bits digits are u_pos = d_pos + 2^(bits-1), and its bits
// above position bits*(NS-1) are the top digit. Zero, and every element of a
// row holding a NaN or an infinity (e == INT32_MAX), get X = 0: all digits 0.
// Halves round up. U is uint64 (bits*NS <= 62) or unsigned __int128.
template <int NS, typename U>
__host__ __device__ __forceinline__ U offset_digits(double v, int e) {
  constexpr int bits = kDigitBits, half = 1 << (bits - 1);
  U H = 0;
#pragma unroll
  for (int pos = 0; pos < NS - 1; ++pos) H |= (U)half << (bits * pos);
  const unsigned long long ab = abs_bits(v);
  const unsigned long long frac = ab & ((1ull << 52) - 1);
  const int be = (int)(ab >> 52);
  const unsigned long long M = be ? (frac | (1ull << 52)) : frac;
  const int E = be ? be - 1075 : -1074;  // |v| = M * 2^E
  const int sh = E - e + bits * NS;
  U X;
  if (e == INT32_MAX) X = 0;
  else if (sh >= 0) X = (U)M << sh;
  else if (sh > -64) X = (U)((M >> (-sh)) + ((M >> (-sh - 1)) & 1ull));
  else X = 0;
  return X + H;
}

// |v| 2^-e for the bound: as bf16 rounded toward zero (0 below bf16's normal
// range: the lower bound only loses that term), and as ceil(|v| 2^(40 - e)),
// an upward-rounded fixed-point term of the row sum. Integer arithmetic on
// the bit pattern only. Rows holding a NaN or an infinity (e == INT32_MAX)
// give 0: their results are NaN and need no bound. With `indicator`, *bf is
// 1.0 for every element that is nonzero (in a finite row), else 0.
__host__ __device__ __forceinline__ void magnitude(double v, int e, bool indicator, uint16_t* bf,
                                                   unsigned long long* fix) {
  *bf = 0;
  *fix = 0;
  const unsigned long long ab = abs_bits(v);
  if (ab == 0 || e == INT32_MAX || ab >= 0x7ff0000000000000ull) return;
  if (indicator) {
    *bf = 0x3f80;  // 1.0
    return;
  }
  const int be = (int)(ab >> 52);
  if (be != 0 && be - 1023 - e <= -1) {
    // normal v below 2^e (every element of a row but subnormals):
    // |v| 2^-e in [2^X, 2^(X+1)) with X = be - 1023 - e. The bf16's 7
    // fraction bits are the top of v's fraction, and |v| 2^(40-e) =
    // M 2^-(12-X) is a right shift by at least 13: the general steps below,
    // with the shift counts known.
    const int X = be - 1023 - e;
    if (X + 127 >= 1) *bf = (uint16_t)(((unsigned)(X + 127) << 7) | ((unsigned)(ab >> 45) & 0x7fu));
    const int r = 12 - X;
    const unsigned long long M = (ab & ((1ull << 52) - 1)) | (1ull << 52);
    *fix = r < 64 ? (M >> r) + ((M << (64 - r)) != 0 ? 1ull : 0ull) : 1ull;
    return;
  }
  const unsigned long long M = be ? ((ab & ((1ull << 52) - 1)) | (1ull << 52)) : ab;
  const int E = be ? be - 1075 : -1074;  // |v| = M 2^E
  const int nb = 64 - clz64(M);          // significant bits of M
  const int X = E - e + nb - 1;          // |v| 2^-e in [2^X, 2^(X+1)), X <= -1
  if (X + 127 >= 1) {
    const unsigned top = (unsigned)(nb >= 8 ? (M >> (nb - 8)) : (M << (8 - nb)));  // leading 8 bits
    *bf = (uint16_t)(((unsigned)(X + 127) << 7) | (top & 0x7fu));
  }
  const int sh = E - e + 40;  // |v| 2^(40-e) = M 2^sh < 2^40
  if (sh >= 0) *fix = M << sh;
  else if (sh > -64) *fix = (M >> (-sh)) + ((M & ((1ull << (-sh)) - 1)) ? 1ull : 0ull);
  else *fix = 1ull;
}

}  // namespace elem
}  // namespace momms
