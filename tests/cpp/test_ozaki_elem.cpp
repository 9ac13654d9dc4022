// Host harness for momms_gb300/csrc/ozaki_elem.cuh: reads cases from stdin,
// one per line (v as its 64-bit pattern), and prints what the functions give.
//   0 vbits                    exponent_of_max(abs_bits(v))
//   1 vbits e ns               offset_digits<ns>(v, e) as "hi lo" (128-bit Y)
//   2 vbits e indicator        magnitude(v, e, indicator) as "bf fix"
#include <stdio.h>
#include <string.h>

#include <type_traits>

#include "ozaki_elem.cuh"

using namespace momms::elem;

template <int NS>
static void digits(double v, int e, unsigned long long* hi, unsigned long long* lo) {
  using U = typename std::conditional<(kDigitBits * NS <= 62), unsigned long long, unsigned __int128>::type;
  const U y = offset_digits<NS, U>(v, e);
  *lo = (unsigned long long)y;
  *hi = (unsigned long long)((unsigned __int128)y >> 64);
}

int main() {
  int kind;
  while (scanf("%d", &kind) == 1) {
    unsigned long long vb;
    if (scanf("%llu", &vb) != 1) return 1;
    double v;
    memcpy(&v, &vb, sizeof v);
    if (kind == 0) {
      printf("%d\n", exponent_of_max(abs_bits(v)));
    } else if (kind == 1) {
      int e, ns;
      if (scanf("%d %d", &e, &ns) != 2) return 1;
      unsigned long long hi = 0, lo = 0;
      switch (ns) {
#define NS_CASE(N) \
  case N: digits<N>(v, e, &hi, &lo); break;
        NS_CASE(1) NS_CASE(2) NS_CASE(3) NS_CASE(4) NS_CASE(5) NS_CASE(6) NS_CASE(7) NS_CASE(8)
        NS_CASE(9) NS_CASE(10) NS_CASE(11) NS_CASE(12) NS_CASE(13) NS_CASE(14) NS_CASE(15)
#undef NS_CASE
        default: return 1;
      }
      printf("%llu %llu\n", hi, lo);
    } else {
      int e, ind;
      if (scanf("%d %d", &e, &ind) != 2) return 1;
      uint16_t bf;
      unsigned long long fix;
      magnitude(v, e, ind != 0, &bf, &fix);
      printf("%u %llu\n", (unsigned)bf, fix);
    }
  }
  return 0;
}
