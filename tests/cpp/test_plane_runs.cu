// Host-side check of the operand passes' run layout (planes.cuh): for every
// block and thread of the grid that planes::run_grid gives, with the lanes
// per row that planes::run_lanes_log2 picks, the rows and runs from
// planes::run_place / planes::run_col and the kernels' row and run loops must
// cover every (row, column) of R x round_up(K, RUN) exactly once, every run
// must start at a multiple of RUN and end inside the padded row, and no
// thread may touch a row past R. Grids whose y extent is cut short exercise
// the kernels' loop over further row chunks. Runs on the CPU: no kernel is
// launched.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "planes.cuh"

using namespace momms::planes;

static int fails = 0;

template <bool R_CONTIG>
static void check(int64_t R, int64_t K, int run, int cap, unsigned ylimit) {
  const int lg = run_lanes_log2(K, run, R_CONTIG, cap);
  dim3 grid = run_grid<R_CONTIG, 8>(R, K, lg);
  if (run != 8) grid = run_grid<R_CONTIG, 4>(R, K, lg);
  if (grid.y > ylimit) grid.y = ylimit;
  const int64_t ldp = (K + run - 1) / run * run;
  std::vector<unsigned char> seen((size_t)(R * ldp), 0);
  for (unsigned by = 0; by < grid.y; ++by)
    for (unsigned bx = 0; bx < grid.x; ++bx)
      for (int tid = 0; tid < THREADS; ++tid) {
        const RunPlace c = run_place<R_CONTIG>(tid, lg);
        for (int64_t r = (int64_t)by * c.rows + c.rl; r < R; r += (int64_t)grid.y * c.rows) {
          for (int it = 0; it < PITER; ++it) {
            const int64_t p = run_col(bx, c, it, run);
            if (p >= K) break;
            if (p % run || p + run > ldp) {
              std::printf("FAIL run R=%lld K=%lld p=%lld\n", (long long)R, (long long)K, (long long)p);
              ++fails;
              return;
            }
            for (int i = 0; i < run; ++i) ++seen[(size_t)(r * ldp + p + i)];
          }
        }
      }
  for (size_t e = 0; e < seen.size(); ++e)
    if (seen[e] != 1) {
      std::printf("FAIL cover R=%lld K=%lld run=%d contig=%d cap=%d ylimit=%u entry=%zu count=%d\n",
                  (long long)R, (long long)K, run, (int)R_CONTIG, cap, ylimit, e, (int)seen[e]);
      ++fails;
      return;
    }
}

int main() {
  const long long shapes[][2] = {{1, 1},   {5, 7},     {33, 64},  {100, 300}, {64, 1025},
                                 {31, 9},  {257, 2049}, {7, 8191}, {70, 40},   {300, 5}};
  for (const auto& s : shapes)
    for (int run : {8, 4})
      for (int cap : {2, 3})
        for (unsigned ylimit : {65535u, 3u}) {
          check<true>(s[0], s[1], run, cap, ylimit);
          check<false>(s[0], s[1], run, cap, ylimit);
        }
  if (fails) return 1;
  std::printf("OK\n");
  return 0;
}
