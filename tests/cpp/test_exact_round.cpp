// Host harness for momms_gb300/csrc/exact_round.cuh: reads cases from stdin,
// one per line, and prints the bits of each double it forms.
//   0 hi lo scale              i128_to_double(hi, lo, scale)
//   1 P0 P1 P2 P3 scale        wide_to_double(P0, P1, P2, P3, scale)
#include <stdio.h>

#include "exact_round.cuh"

int main() {
  int kind;
  while (scanf("%d", &kind) == 1) {
    double v;
    int sc;
    if (kind == 0) {
      long long hi;
      unsigned long long lo;
      if (scanf("%lld %llu %d", &hi, &lo, &sc) != 3) return 1;
      v = momms::i128_to_double(hi, lo, sc);
    } else {
      long long p0, p1, p2, p3;
      if (scanf("%lld %lld %lld %lld %d", &p0, &p1, &p2, &p3, &sc) != 5) return 1;
      v = momms::wide_to_double(p0, p1, p2, p3, sc);
    }
    unsigned long long b;
    memcpy(&b, &v, sizeof(b));
    printf("%llu\n", b);
  }
  return 0;
}
