// Per-shape launch configuration: the runtime analogue of the reference's
// compile-time block sizes (the typenum NC/KC/MC/MR/NR of
// src/exper/l3_packing.rs:58-66). A configuration depends only on
// (dtype, precision, m, n, k) and the device's SM count, never on what else is
// in a batch, so a problem gives the same bits alone and in any mix.
//
// The split-k count comes from a measured table filled by momms_autotune()
// (candidates timed with CUDA events on scratch output) or, for shapes not in
// the table, from a model: split k only when the output tiles cannot fill the
// GPU, keeping at least 2 (f64, 32 of k) / 8 (f32, 128 of k) k-blocks per split.
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"

namespace momms {

namespace {
typedef std::tuple<int, int, int64_t, int64_t, int64_t> Key;  // dtype, precision, m, n, k
std::mutex g_tmu;
std::map<Key, int> g_table;  // -> splits
thread_local int g_force_splits = 0;  // set while the tuner times a candidate

int model_splits(int64_t tiles, int64_t kblocks, int slots, int64_t min_kb) {
  int splits = 1;
  if (tiles < slots) {
    splits = (int)std::min<int64_t>(slots / tiles, kblocks / min_kb);
    splits = std::max(1, std::min(splits, 32));
  }
  return splits;
}

int lookup(int dtype, int prec, int64_t m, int64_t n, int64_t k) {
  if (g_force_splits > 0) return g_force_splits;
  std::lock_guard<std::mutex> lk(g_tmu);
  auto it = g_table.find(Key{dtype, prec, m, n, k});
  return it == g_table.end() ? 0 : it->second;
}
}  // namespace

int splits_f64(int64_t m, int64_t n, int64_t k, int sm_count) {
  const int64_t tiles = ceil_div(m, 128) * ceil_div(n, 128), kblocks = ceil_div(k, 16);
  int s = lookup(MOMMS_DTYPE_F64, MOMMS_PREC_PLAIN, m, n, k);
  // Small problems: one SM's FP64 rate is ~7 GFLOP/s, so splitting k down to
  // two k-blocks (32) per unit beats leaving SMs idle. Measured on GB300 with
  // the dynamically scheduled grouped kernel: 256^3 0.33 -> 0.21 ms and 128^3
  // 0.32 -> 0.19 ms against four k-blocks per unit, while a batch of 239 small
  // f64 problems, whose splits' fixed costs (pipeline fill, partial write,
  // reduction) buy no parallelism, took 3 % longer (14.2 -> 14.7 ms); one
  // k-block per unit gained 256^3 another 20 % but cost the batch 8 %.
  if (s <= 0) s = model_splits(tiles, kblocks, sm_count, 2);
  return std::max(1, (int)std::min<int64_t>(s, std::max<int64_t>(1, kblocks)));
}

int splits_f32(int64_t m, int64_t n, int64_t k, int sm_count) {
  const int64_t tiles = ceil_div(m, 128) * ceil_div(n, 128), kblocks = ceil_div(k, 16);
  int s = lookup(MOMMS_DTYPE_F32, MOMMS_PREC_PLAIN, m, n, k);
  if (s <= 0) s = model_splits(tiles, kblocks, 2 * sm_count, 8);
  return std::max(1, (int)std::min<int64_t>(s, std::max<int64_t>(1, kblocks)));
}

}  // namespace momms

extern "C" {

int momms_autotune(const momms_gemm_desc* desc, momms_tune_result* out, void* stream) {
  using namespace momms;
  if (!desc) return fail(MOMMS_ERR_INVALID_ARG, "desc is null");
  int rc = momms_gemm_validate(desc);
  if (rc) return rc;
  if (desc->precision != MOMMS_PREC_PLAIN)
    return fail(MOMMS_ERR_UNSUPPORTED, "autotuning covers the plain paths (split-k); other modes plan per call");
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
  const int cands[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32};
  int best = 1;
  float best_ms = 1e30f;
  int tried = 0;
  for (int c : cands) {
    if (c > 1 && kblocks / c < 2) break;
    g_force_splits = c;
    float ms_sum = 0.f;
    int reps = 3;
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
    g_force_splits = 0;
    if (rc) break;
    ++tried;
    if (ms_sum / reps < best_ms) {
      best_ms = ms_sum / reps;
      best = c;
    }
  }
  g_force_splits = 0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(cs);
  if (rc) return rc;
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    g_table[Key{desc->dtype, desc->precision, desc->m, desc->n, desc->k}] = best;
  }
  if (out) {
    out->splits = best;
    out->candidates = tried;
    out->best_ms = best_ms;
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
      snprintf(line, sizeof(line), "%d %d %lld %lld %lld %d\n", std::get<0>(kv.first), std::get<1>(kv.first),
               (long long)std::get<2>(kv.first), (long long)std::get<3>(kv.first), (long long)std::get<4>(kv.first),
               kv.second);
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
  std::vector<std::pair<Key, int>> rows;
  const char* p = text;
  while (*p) {
    int dt, pr, sp;
    long long m, n, k;
    int used = 0;
    if (sscanf(p, "%d %d %lld %lld %lld %d%n", &dt, &pr, &m, &n, &k, &sp, &used) != 6)
      return fail(MOMMS_ERR_INVALID_ARG, "malformed tuning line near '%.20s'", p);
    if (dt < 0 || dt > 1 || pr < 0 || pr > 2 || m <= 0 || n <= 0 || k <= 0 || sp < 1 || sp > 32)
      return fail(MOMMS_ERR_INVALID_ARG, "tuning line out of range near '%.20s'", p);
    rows.push_back({Key{dt, pr, m, n, k}, sp});
    p += used;
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
