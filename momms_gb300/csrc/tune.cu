// Per-shape launch configuration of the plain paths: the runtime analogue of
// the reference's compile-time block sizes (the typenum NC/KC/MC/MR/NR of
// src/exper/l3_packing.rs:58-66). A configuration is an output tile (the
// kernel's large tile or its small one) and a k-split count. It depends only
// on (dtype, precision, m, n, k) and the device's SM count, never on what else
// is in a batch, so a problem gives the same bits alone and in any mix.
//
// The table that momms_autotune fills (candidates timed with CUDA events on a
// scratch output) is keyed by shape bucket: ceil(log2) of m, n and k, so a
// tuned shape covers every problem within a factor of two of it and a batch
// of uneven problems hits tuned entries. Shapes without an entry use a model:
// the large tile, and k split only while the tiles leave CTA slots idle,
// keeping at least 2 (f64, 32 of k) / 8 (f32, 128 of k) k-blocks per split.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"

namespace momms {

namespace {
typedef std::tuple<int, int, int, int, int> Key;  // dtype, precision, lg m, lg n, lg k
std::mutex g_tmu;
std::map<Key, PlainCfg> g_table;
thread_local PlainCfg g_force = {-1, 0};  // set while the tuner times a candidate

int lg_ceil(int64_t x) {
  int b = 0;
  while (b < 62 && ((int64_t)1 << b) < x) ++b;
  return b;
}
Key key_of(int dtype, int prec, int64_t m, int64_t n, int64_t k) {
  return Key{dtype, prec, lg_ceil(m), lg_ceil(n), lg_ceil(k)};
}

int model_splits(int64_t tiles, int64_t kblocks, int64_t slots, int64_t min_kb) {
  int splits = 1;
  if (tiles < slots) {
    splits = (int)std::min<int64_t>(slots / tiles, kblocks / min_kb);
    splits = std::max(1, std::min(splits, 32));
  }
  return splits;
}

bool lookup(int dtype, int prec, int64_t m, int64_t n, int64_t k, PlainCfg* out) {
  if (g_force.tile >= 0) {
    *out = g_force;
    return true;
  }
  std::lock_guard<std::mutex> lk(g_tmu);
  auto it = g_table.find(key_of(dtype, prec, m, n, k));
  if (it == g_table.end()) return false;
  *out = it->second;
  return true;
}

int clamp_splits(int s, int64_t kblocks) { return std::max(1, (int)std::min<int64_t>(s, std::max<int64_t>(1, kblocks))); }
}  // namespace

PlainCfg plain_cfg(int dtype, int64_t m, int64_t n, int64_t k, int sm_count) {
  const int64_t kblocks = ceil_div(k, 16);
  PlainCfg c;
  if (lookup(dtype, MOMMS_PREC_PLAIN, m, n, k, &c)) {
    c.splits = clamp_splits(c.splits, kblocks);
    return c;
  }
  if (dtype == MOMMS_DTYPE_F64) {
    // Small problems: one SM's FP64 rate is ~7 GFLOP/s, so splitting k down
    // to two k-blocks (32) per unit beats leaving SMs idle. Measured on
    // GB300 with the dynamically scheduled grouped kernel: 256^3 0.33 ->
    // 0.21 ms and 128^3 0.32 -> 0.19 ms against four k-blocks per unit, while
    // a batch of 239 small f64 problems, whose splits' fixed costs (pipeline
    // fill, partial write, reduction) buy no parallelism, took 3 % longer
    // (14.2 -> 14.7 ms); one k-block per unit gained 256^3 another 20 % but
    // cost the batch 8 %.
    const int64_t tiles = ceil_div(m, 128) * ceil_div(n, 128);
    c.tile = 0;
    c.splits = clamp_splits(model_splits(tiles, kblocks, sm_count, 2), kblocks);
    return c;
  }
  // f32: the 128 x 128 tile (two CTAs per SM), split while its tiles leave
  // CTA slots idle. The 64 x 64 tile is chosen only by the tuner: as the
  // model's choice for every shape whose large tiles leave slots idle it took
  // the f32 part of the 512-problem batch from 0.65 to 0.85 ms (a second
  // persistent launch per batch, and no faster per problem there).
  const int64_t tiles128 = ceil_div(m, 128) * ceil_div(n, 128);
  c.tile = 0;
  c.splits = clamp_splits(model_splits(tiles128, kblocks, 2 * (int64_t)sm_count, 8), kblocks);
  return c;
}

int splits_f64(int64_t m, int64_t n, int64_t k, int sm_count) { return plain_cfg(MOMMS_DTYPE_F64, m, n, k, sm_count).splits; }

}  // namespace momms

extern "C" {

int momms_autotune(const momms_gemm_desc* desc, momms_tune_result* out, void* stream) {
  using namespace momms;
  if (!desc) return fail(MOMMS_ERR_INVALID_ARG, "desc is null");
  int rc = momms_gemm_validate(desc);
  if (rc) return rc;
  if (desc->precision != MOMMS_PREC_PLAIN)
    return fail(MOMMS_ERR_UNSUPPORTED, "autotuning covers the plain paths (tile, split-k); other modes plan per call");
  if (desc->m == 0 || desc->n == 0 || desc->k == 0) return fail(MOMMS_ERR_INVALID_ARG, "empty problem");
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t es = desc->dtype == MOMMS_DTYPE_F64 ? 8 : 4;
  const int bk = 16;  // k-block of both the DMMA and the FFMA kernels
  const int64_t kblocks = ceil_div(desc->k, bk);
  // scratch C so that the caller's C is not touched
  void* cs = nullptr;
  cudaError_t e = device_malloc((void**)&cs, (size_t)desc->m * desc->n * es);
  if (e != cudaSuccess) return cuda_fail(e, "autotune scratch");
  momms_gemm_desc d = *desc;
  d.c = momms_operand{cs, 1, desc->m, MOMMS_MEM_DEVICE, 0};
  d.beta = 0.0;
  d.a.mem = d.b.mem = MOMMS_MEM_DEVICE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // candidates: each tile the dtype's kernel has, with the split counts that
  // keep at least two k-blocks per split
  const int split_cands[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32};
  const int ntiles = desc->dtype == MOMMS_DTYPE_F32 ? 2 : 1;
  PlainCfg best = {0, 1};
  float best_ms = 1e30f;
  int tried = 0;
  for (int tile = 0; tile < ntiles && !rc; ++tile) {
    for (int c : split_cands) {
      if (c > 1 && kblocks / c < 2) break;
      g_force = PlainCfg{tile, c};
      float ms_sum = 0.f;
      const int reps = 3;
      rc = momms_gemm(&d, stream);  // warm-up
      for (int r = 0; r < reps && !rc; ++r) {
        cudaEventRecord(e0, s);
        rc = momms_gemm(&d, stream);
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_sum += ms;
      }
      g_force = PlainCfg{-1, 0};
      if (rc) break;
      ++tried;
      if (ms_sum / reps < best_ms) {
        best_ms = ms_sum / reps;
        best = PlainCfg{tile, c};
      }
    }
  }
  g_force = PlainCfg{-1, 0};
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(cs);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    g_table[key_of(desc->dtype, desc->precision, desc->m, desc->n, desc->k)] = best;
  }
  if (out) {
    out->splits = best.splits;
    out->candidates = tried;
    out->best_ms = best_ms;
    out->tile = best.tile;
  }
  return MOMMS_OK;
}

int momms_autotune_batch(const momms_gemm_desc* descs, int count, void* stream, int* tuned) {
  using namespace momms;
  if (tuned) *tuned = 0;
  if (!descs || count < 0) return fail(MOMMS_ERR_INVALID_ARG, "bad batch");
  std::set<Key> seen;
  for (int i = 0; i < count; ++i) {
    const momms_gemm_desc& d = descs[i];
    if (d.precision != MOMMS_PREC_PLAIN || d.m == 0 || d.n == 0 || d.k == 0) continue;
    const Key key = key_of(d.dtype, d.precision, d.m, d.n, d.k);
    if (!seen.insert(key).second) continue;  // the bucket's first problem stands for it
    const int rc = momms_autotune(&d, nullptr, stream);
    if (rc) return rc;
    if (tuned) *tuned += 1;
  }
  return MOMMS_OK;
}

int momms_tune_export(char* buf, size_t cap, size_t* needed) {
  using namespace momms;
  std::string text;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    char line[160];
    for (const auto& kv : g_table) {
      // a bucket is written as its largest shape
      snprintf(line, sizeof(line), "%d %d %lld %lld %lld %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
               1ll << std::get<2>(kv.first), 1ll << std::get<3>(kv.first), 1ll << std::get<4>(kv.first),
               kv.second.splits, kv.second.tile);
      text += line;
    }
  }
  if (needed) *needed = text.size() + 1;
  if (buf && cap > 0) {
    const size_t n = std::min(cap - 1, text.size());
    memcpy(buf, text.data(), n);
    buf[n] = 0;
    if (cap < text.size() + 1) return fail(MOMMS_ERR_INVALID_ARG, "buffer too small (%zu bytes needed)", text.size() + 1);
  }
  return MOMMS_OK;
}

int momms_tune_import(const char* text) {
  using namespace momms;
  if (!text) return fail(MOMMS_ERR_INVALID_ARG, "text is null");
  std::vector<std::pair<Key, PlainCfg>> rows;
  const char* p = text;
  while (*p) {
    int dt, pr, sp, tile = 0;
    long long m, n, k;
    int used = 0;
    if (sscanf(p, "%d %d %lld %lld %lld %d%n", &dt, &pr, &m, &n, &k, &sp, &used) != 6)
      return fail(MOMMS_ERR_INVALID_ARG, "malformed tuning line near '%.20s'", p);
    p += used;
    // optional seventh field on the same line: the tile
    const char* q = p;
    while (*q == ' ' || *q == '\t') ++q;
    if (*q >= '0' && *q <= '9') {
      int used2 = 0;
      if (sscanf(q, "%d%n", &tile, &used2) != 1) return fail(MOMMS_ERR_INVALID_ARG, "malformed tile near '%.20s'", q);
      p = q + used2;
    }
    if (dt < 0 || dt > 1 || pr != MOMMS_PREC_PLAIN || m <= 0 || n <= 0 || k <= 0 || sp < 1 || sp > 32 || tile < 0 ||
        tile > (dt == MOMMS_DTYPE_F32 ? 1 : 0))
      return fail(MOMMS_ERR_INVALID_ARG, "tuning line out of range near '%.20s'", text);
    rows.push_back({key_of(dt, pr, m, n, k), PlainCfg{tile, sp}});
    while (*p == '\n' || *p == ' ' || *p == '\r' || *p == '\t') ++p;
  }
  std::lock_guard<std::mutex> lk(g_tmu);
  for (auto& r : rows) g_table[r.first] = r.second;
  return MOMMS_OK;
}

int momms_tune_clear(void) {
  std::lock_guard<std::mutex> lk(momms::g_tmu);
  momms::g_table.clear();
  return MOMMS_OK;
}

}  // extern "C"
