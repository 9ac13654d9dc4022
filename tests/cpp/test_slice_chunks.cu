// Host-side check of the slice kernels' TMEM chunk plan: sp::plan_chunks'
// closed-form chunk count per group must equal the count the MMA issuer
// produces step by step (close a chunk before a (pair, k-block) step whose
// weight would pass chunk_cap, or at a pair boundary without merge_pairs).
// Runs on the CPU: no kernel is instantiated or launched.
#include <cstdio>
#include <cstdlib>

#include "slicegemm.cuh"

using momms::sp::Params;

static int issuer_count(const Params& p, int g) {
  int n = 0, load = 0;
  bool open = false;
  for (int pp = p.group_begin[g]; pp < p.group_begin[g + 1]; ++pp) {
    const int w = p.pair_w[pp];
    for (int st = 0; st < p.kblocks; ++st) {
      if (open && (load + w > p.chunk_cap || (st == 0 && !p.merge_pairs))) open = false;
      if (!open) {
        ++n;
        load = 0;
        open = true;
      }
      load += w;
    }
  }
  return n;
}

int main() {
  static Params p;
  unsigned seed = 12345u;
  auto rnd = [&](int lo, int hi) {  // inclusive
    seed = seed * 1664525u + 1013904223u;
    return lo + (int)((seed >> 8) % (unsigned)(hi - lo + 1));
  };
  for (int trial = 0; trial < 20000; ++trial) {
    const int caps[] = {8, 16, 256, 7, 13};
    p.chunk_cap = caps[rnd(0, 4)];
    p.merge_pairs = rnd(0, 1);
    p.kblocks = rnd(1, 600);
    p.ngroups = rnd(1, 12);
    int np = 0;
    for (int g = 0; g < p.ngroups; ++g) {
      p.group_begin[g] = np;
      const int pairs = rnd(1, 8);
      for (int i = 0; i < pairs; ++i) p.pair_w[np++] = rnd(1, p.chunk_cap);
    }
    p.group_begin[p.ngroups] = np;
    if (!momms::sp::plan_chunks(p)) {
      printf("plan_chunks rejected valid weights\n");
      return 1;
    }
    for (int g = 0; g < p.ngroups; ++g) {
      const int want = issuer_count(p, g);
      if (p.group_chunks[g] != want) {
        printf("trial %d group %d: planned %d chunks, issuer %d\n", trial, g, p.group_chunks[g], want);
        return 1;
      }
    }
  }
  // a weight above the capacity is refused
  p.ngroups = 1;
  p.group_begin[0] = 0;
  p.group_begin[1] = 1;
  p.pair_w[0] = 17;
  p.chunk_cap = 16;
  if (momms::sp::plan_chunks(p)) {
    printf("plan_chunks accepted a weight above the capacity\n");
    return 1;
  }
  // the Ozaki weights at 8-bit digits: a lone pair's chunk is 4, 8 or 16 k-blocks
  p.chunk_cap = 256;
  p.merge_pairs = 1;
  p.kblocks = 128;
  p.ngroups = 3;
  p.group_begin[0] = 0; p.group_begin[1] = 1; p.group_begin[2] = 2; p.group_begin[3] = 3;
  p.pair_w[0] = 64; p.pair_w[1] = 32; p.pair_w[2] = 16;
  if (!momms::sp::plan_chunks(p) || p.group_chunks[0] != 32 || p.group_chunks[1] != 16 || p.group_chunks[2] != 8) {
    printf("Ozaki chunk lengths wrong: %d %d %d\n", p.group_chunks[0], p.group_chunks[1], p.group_chunks[2]);
    return 1;
  }
  printf("OK\n");
  return 0;
}
