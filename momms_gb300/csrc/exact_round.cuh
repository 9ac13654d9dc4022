// Exact integer -> double rounding of the Ozaki recombination: the nearest
// double (ties to even) to a 128-bit or wider integer times a power of two,
// in integer instructions only. Host and device code: the CPU tests compile
// this header with the host compiler and compare every result with exact
// rational rounding.
#pragma once
#include <string.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace momms {

__host__ __device__ __forceinline__ int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// Nearest double (ties to even) to (hi 2^64 + lo) * 2^scale, hi:lo a 128-bit
// two's complement integer other than -2^127. The magnitude is normalised
// to bit 127 first, so one 64-bit word holds the 53 bits kept and the
// rounding bit, and the word below only feeds the sticky test: integer
// instructions only, since GB300's FP64 pipe is narrow, and no branch on
// the operand's size. Subnormal results are rounded once, at their own
// quantum; results past the largest double are infinite.
__host__ __device__ __forceinline__ double i128_to_double(long long hi_s, unsigned long long lo, int scale) {
  const bool neg = hi_s < 0;
  unsigned long long hi = (unsigned long long)hi_s;
  if (neg) {  // two's complement negation of hi:lo
    lo = 0ull - lo;
    hi = ~hi + (lo == 0 ? 1ull : 0ull);
  }
  if ((hi | lo) == 0) return 0.0;
  const int lz = hi ? clz64(hi) : 64 + clz64(lo);
  unsigned long long nh, nl;  // |R| << lz: bit 63 of nh set
  if (lz >= 64) {
    nh = lo << (lz - 64);
    nl = 0;
  } else {
    nh = lz ? (hi << lz) | (lo >> (64 - lz)) : hi;
    nl = lo << lz;
  }
  unsigned long long mant = nh >> 11;  // 53 bits
  const unsigned rb = (unsigned)(nh & 0x7ffull);
  if (rb > 0x400u || (rb == 0x400u && (nl != 0 || (mant & 1ull)))) ++mant;
  int E = 127 - lz + scale;  // value = (mant / 2^52) * 2^E
  if (mant >> 53) {
    mant >>= 1;
    ++E;
  }
  const unsigned long long sign = neg ? (1ull << 63) : 0ull;
  unsigned long long b;
  if (E > 1023) {
    b = sign | (0x7ffull << 52);  // past the largest double: infinity
  } else if (E >= -1022) {
    b = sign | ((unsigned long long)(E + 1023) << 52) | (mant & ((1ull << 52) - 1));
  } else {
    // subnormal: round nh:nl once at the quantum 2^-1074, bit sh of nh
    // (nh's bit 63 weighs 2^E before the rounding above)
    E = 127 - lz + scale;
    const int sh = -1011 - E;  // >= 12
    unsigned long long m = 0;
    if (sh < 64) {
      m = nh >> sh;
      const unsigned long long half = 1ull << (sh - 1), rem = nh & ((1ull << sh) - 1);
      if (rem > half || (rem == half && (nl != 0 || (m & 1ull)))) ++m;
    } else if (sh == 64 && ((nh << 1) != 0 || nl != 0)) {
      m = 1;  // above half the quantum
    }
    b = sign | m;  // m = 2^52 is the smallest normal number
  }
  double r;
  memcpy(&r, &b, sizeof(r));
  return r;
}

__host__ __device__ __forceinline__ double i128_to_double(__int128 R, int scale) {
  return i128_to_double((long long)(R >> 64), (unsigned long long)R, scale);
}

// Nearest double to R * 2^scale, R = P0 + P1 2^32 + P2 2^64 + P3 2^96 exactly
// (|R| < 2^148). R below 2^126 in magnitude goes through i128_to_double as
// is; a wider R is first shifted right to 126 bits with the lost bits kept
// as a sticky bit 0 (more than the 53 + 2 bits the rounding looks at), which
// leaves the rounded result unchanged.
__host__ __device__ __forceinline__ double wide_to_double(long long P0, long long P1, long long P2, long long P3, int scale) {
  const __int128 low = (__int128)P0 + ((__int128)P1 << 32);        // |.| < 2^93
  const __int128 hi = (__int128)P2 + ((__int128)P3 << 32) + (low >> 64);  // R = hi 2^64 + lo, lo in [0, 2^64)
  const unsigned long long lo = (unsigned long long)low;
  const __int128 lim = (__int128)1 << 61;
  if (hi >= -lim && hi < lim) return i128_to_double((__int128)(((unsigned __int128)hi << 64) | lo), scale);
  const bool neg = hi < 0;
  // the magnitude as uh 2^64 + ul
  unsigned __int128 uh = neg ? (unsigned __int128)(-hi) - (lo != 0 ? 1u : 0u) : (unsigned __int128)hi;
  const unsigned long long ul = neg ? (0ull - lo) : lo;
  const unsigned long long uh_hi = (unsigned long long)(uh >> 64), uh_lo = (unsigned long long)uh;
  const int nbh = uh_hi ? 128 - clz64(uh_hi) : 64 - clz64(uh_lo);  // bits of uh (>= 62)
  const int s = nbh + 64 - 126;  // 1..22: the magnitude has nbh + 64 bits
  unsigned __int128 u = (uh << (64 - s)) | (unsigned __int128)(ul >> s);
  if (ul & ((1ull << s) - 1)) u |= 1u;  // sticky
  return i128_to_double(neg ? -(__int128)u : (__int128)u, scale + s);
}

}  // namespace momms
