// Grouped persistent launches: many independent GEMMs in one kernel per
// dtype, and the execution plans (momms_plan_*) that hold their problem
// tables, workspaces and an optional CUDA graph.
//
// Every plain f64 problem contributes tiles x splits work units to one
// persistent DMMA kernel and every plain f32 problem to one persistent FFMA
// kernel. Units are ordered by decreasing cost (longest first) and handed to
// the CTAs through a global atomic counter. Each problem keeps the split
// count a single launch of its shape uses (the tuning table or the model,
// tune.cu: the runtime analogue of the reference's compile-time block
// sizes), and its k-splits are reduced in a fixed order, so a problem's
// result does not depend on the rest of the batch.
#include <string.h>

#include <algorithm>
#include <mutex>
#include <numeric>
#include <vector>

#include "dmma_core.cuh"
#include "ffma_core.cuh"
#include "internal.h"

namespace momms {
namespace grouped {

struct DProblem {
  int64_t m, n, k;
  double alpha, beta;
  double* c;
  int64_t rsc, csc;
  int tiles_m, tiles_n, splits, flags;  // flags: bit 0 A x-contiguous, bit 1 B x-contiguous
  int64_t kb_split;
  int64_t unit_begin;
  int64_t part_offset;     // elements into the partials buffer
  int64_t counter_offset;  // entries into the counters buffer
};

struct SProblem {
  ffma::Operands o;
  ffma::Epi e;
  int tiles_m, tiles_n, splits, pad;
  int64_t kb_split;
  int64_t unit_begin;
  int64_t part_offset;
  int64_t counter_offset;
};

template <typename P>
__device__ __forceinline__ int find_problem(const P* probs, int nprobs, int64_t u) {
  int lo = 0, hi = nprobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].unit_begin <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Decodes unit u of the f64 group: its problem, output tile and k-blocks.
struct DUnit {
  int pi, tm, tn, sp;
  int64_t tile, kb0, kb1;
};
__device__ __forceinline__ DUnit decode_dunit(const DProblem* probs, int nprobs, int64_t u) {
  using namespace dmma;
  DUnit d;
  d.pi = find_problem(probs, nprobs, u);
  const DProblem& P = probs[d.pi];
  const int64_t local = u - P.unit_begin;
  d.sp = (int)(local % P.splits);
  d.tile = local / P.splits;
  d.tm = (int)(d.tile % P.tiles_m);
  d.tn = (int)(d.tile / P.tiles_m);
  const int64_t kblocks = ceil_div_dev(P.k, BK);
  d.kb0 = d.sp * P.kb_split;
  d.kb1 = min(kblocks, d.kb0 + P.kb_split);
  return d;
}

// Units are handed out dynamically: the producer lane takes the next unit
// from a global counter (units are numbered largest problem first, so this
// is longest-processing-time-first list scheduling, balanced by the actual
// unit durations rather than a cost model) and tags the first pipeline stage
// it fills for that unit with the unit's index; the DMMA warps read the tag
// when they reach that stage. An index of -1 ends the kernel. The last CTA
// to finish resets the counter, so a captured plan relaunches as is.
__global__ void __launch_bounds__(dmma::THREADS, 1)
    dgemm_grouped_kernel(const CUtensorMap* __restrict__ maps, const DProblem* __restrict__ probs, int nprobs,
                         int64_t total_units, double* partials, unsigned* counters, unsigned long long* next_unit,
                         unsigned* status) {
  using namespace dmma;
  extern __shared__ uint8_t smem_raw[];
  __shared__ long long s_stage_unit[STAGES];  // unit starting at each stage, -1: end
  const Smem sm = setup_smem(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int stage = 0;
  uint32_t phase = 0;
  if (warp == CONSUMER_WARPS) {
    if (lane == 0) {
      bool ok = true;
      for (;;) {
        const long long u = (long long)atomicAdd(next_unit, 1ull);
        if (u >= total_units) break;
        const DUnit d = decode_dunit(probs, nprobs, u);
        const DProblem& P = probs[d.pi];
        // the tag is written while the stage is free (every DMMA warp read
        // the previous tag before releasing it) and published by the
        // stage's arrive (release) to the warps' wait (acquire)
        if (!mbar_wait_bounded(&sm.empty[stage], phase ^ 1)) {
          report_status(status, DEV_TIMEOUT_EMPTY);
          ok = false;
          break;
        }
        s_stage_unit[stage] = u;
        if (!produce_unit(&maps[2 * d.pi], &maps[2 * d.pi + 1], P.flags & 1, (P.flags >> 1) & 1, d.tm, d.tn, d.kb0,
                          d.kb1, sm.sA, sm.sB, sm.full, sm.empty, stage, phase, status)) {
          ok = false;
          break;
        }
      }
      if (ok) {
        if (mbar_wait_bounded(&sm.empty[stage], phase ^ 1)) {
          s_stage_unit[stage] = -1;
          mbar_arrive(&sm.full[stage]);
        } else {
          report_status(status, DEV_TIMEOUT_EMPTY);
        }
      }
      // the last CTA out resets the unit counter for the next launch
      __threadfence();
      const unsigned long long done = atomicAdd(next_unit + 1, 1ull);
      if (done == (unsigned long long)gridDim.x - 1) {
        next_unit[0] = 0ull;
        next_unit[1] = 0ull;
        __threadfence();
      }
    }
    return;
  }
  const int wm = warp >> 2, wn = warp & 3;
  for (;;) {
    if (!mbar_wait_bounded(&sm.full[stage], phase)) {
      report_status(status, DEV_TIMEOUT_FULL);
      return;
    }
    const long long u = s_stage_unit[stage];
    if (u < 0) break;
    const DUnit d = decode_dunit(probs, nprobs, u);
    const DProblem& P = probs[d.pi];
    const int64_t row_base = (int64_t)d.tm * BM + wm * 64, col_base = (int64_t)d.tn * BN + wn * 32;
    const uint32_t live = live_mask(row_base, col_base, P.m, P.n);
    double acc[8][4][2];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;
    if (!consume_unit(P.flags & 1, (P.flags >> 1) & 1, d.kb0, d.kb1, live, sm.sA, sm.sB, sm.full, sm.empty, stage,
                      phase, wm, wn, lane, acc, status))
      return;
    const Epi e{P.m, P.n, P.alpha, P.beta, P.c, P.rsc, P.csc};
    finish_unit(e, acc, row_base + (lane >> 2), col_base + 2 * (lane & 3), P.splits, d.sp,
                P.splits > 1 ? partials + P.part_offset + (size_t)d.tile * P.splits * BM * BN : nullptr,
                P.splits > 1 ? counters + P.counter_offset + d.tile : nullptr, threadIdx.x, sm.s_last);
  }
}

template <int TM, typename Off>
__global__ void __launch_bounds__(ffma::Tile<TM>::THREADS, ffma::Tile<TM>::CTAS_PER_SM)
    sgemm_grouped_kernel(const SProblem* __restrict__ probs, int nprobs, int64_t total_units,
                         unsigned long long* next_unit, float* partials, unsigned* counters) {
  using namespace ffma;
  extern __shared__ float4 ffma_smem[];
  __shared__ int s_last;
  __shared__ long long s_unit;
  for (;;) {
    if (threadIdx.x == 0) s_unit = (long long)atomicAdd(next_unit, 1ull);
    __syncthreads();
    const int64_t u = s_unit;
    __syncthreads();
    if (u >= total_units) break;
    const int pi = find_problem(probs, nprobs, u);
    const SProblem& P = probs[pi];
    const int64_t local = u - P.unit_begin;
    const int sp = (int)(local % P.splits);
    const int64_t tile = local / P.splits;
    const int tm = (int)(tile % P.tiles_m), tn = (int)(tile / P.tiles_m);
    const int64_t kblocks = ceil_div_dev(P.o.k, BK);
    const int64_t kb0 = sp * P.kb_split, kb1 = min(kblocks, kb0 + P.kb_split);
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    prefetch_c_tile<TM>(P.e, tm, tn);
    ffma_unit_any<TM, Off>(P.o, tm, tn, kb0, kb1, acc, reinterpret_cast<float*>(ffma_smem));
    ffma_finish<TM>(P.e, acc, tm, tn, P.splits, sp,
                    P.splits > 1 ? partials + P.part_offset + (size_t)tile * P.splits * TM * TM : nullptr,
                    P.splits > 1 ? counters + P.counter_offset + tile : nullptr, &s_last);
  }
  // the last CTA out resets the unit counter for the next launch of the plan
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long done = atomicAdd(next_unit + 1, 1ull);
    if (done == (unsigned long long)gridDim.x - 1) {
      next_unit[0] = 0ull;
      next_unit[1] = 0ull;
      __threadfence();
    }
  }
}

}  // namespace grouped

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------

struct PlanProblem {
  momms_gemm_desc d;
  int slices;  // Ozaki: frozen slice count
};

struct Plan {
  int device = -1;
  // stream-ordered mode (used by the server): allocations, uploads and frees
  // are enqueued on `stream` instead of synchronising the device
  bool async = false;
  cudaStream_t stream = nullptr;
  std::vector<char> host_tables;  // upload sources, alive until destroy
  // f64 plain group
  int nd = 0;
  int64_t d_units = 0;
  grouped::DProblem* d_probs = nullptr;  // device
  CUtensorMap* d_maps = nullptr;         // device
  double* d_partials = nullptr;
  unsigned* d_counters = nullptr;
  unsigned long long* d_next = nullptr;  // unit counter + finished-CTA counter
  // f32 plain groups, one per FFMA tile (0: 128 x 128, 1: 64 x 64), each
  // one persistent launch
  struct SGroup {
    int ns = 0;
    int64_t units = 0;
    grouped::SProblem* probs = nullptr;
    float* partials = nullptr;
    unsigned* counters = nullptr;
    unsigned long long* next = nullptr;
    bool wide = false;  // some f32 operand needs 64-bit element offsets
  } sg[2];
  // problems run by their own launch sequence (Ozaki, split-TF32)
  std::vector<PlanProblem> other;
  // two or more emulated problems with fixed slice counts: one slice launch
  OzakiBatch* ozb = nullptr;
  // operands copied to column-major scratch before each launch (f64
  // operands whose strides do not suit TMA)
  struct Repack {
    DevMat src;
    int64_t rows, cols;
    void* dst;
    int64_t ld;
  };
  std::vector<Repack> repacks;
  // captured graph
  cudaGraphExec_t graph = nullptr;
  std::vector<void*> allocs;
};

namespace {

int plan_alloc(Plan* p, void** out, size_t bytes) {
  if (bytes == 0) {
    *out = nullptr;
    return MOMMS_OK;
  }
  cudaError_t e = p->async ? scratch_alloc(out, bytes, p->stream) : device_malloc(out, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "plan allocation");
  p->allocs.push_back(*out);
  return MOMMS_OK;
}

void plan_free(Plan* p) {
  if (p->graph) cudaGraphExecDestroy(p->graph);
  ozaki_batch_destroy(p->ozb);
  for (void* a : p->allocs) {
    if (p->async) cudaFreeAsync(a, p->stream);
    else cudaFree(a);
  }
  delete p;
}

bool on_device(const void* ptr) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

int set_attrs_grouped() {
  cudaError_t e = cudaFuncSetAttribute(grouped::dgemm_grouped_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       dmma::SMEM_BYTES);
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "cudaFuncSetAttribute(grouped)");
}

// Copies host bytes to the device: synchronously, or stream-ordered from a
// copy kept in the plan until it is destroyed.
int plan_upload(Plan* p, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return MOMMS_OK;
  cudaError_t e;
  if (p->async) {
    const size_t off = p->host_tables.size();
    p->host_tables.resize(off + bytes);
    memcpy(p->host_tables.data() + off, src, bytes);
    (void)off;
    e = cudaSuccess;
  } else {
    e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  }
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "plan upload");
}

int plan_zero(Plan* p, void* dst, size_t bytes) {
  if (bytes == 0) return MOMMS_OK;
  cudaError_t e = p->async ? cudaMemsetAsync(dst, 0, bytes, p->stream) : cudaMemset(dst, 0, bytes);
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "plan workspace");
}

int plan_create(const momms_gemm_desc* descs, int count, Plan** out, cudaStream_t async_stream, bool async) {
  *out = nullptr;
  if (!descs || count < 0) return fail(MOMMS_ERR_INVALID_ARG, "descs is null or count < 0");
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  for (int i = 0; i < count; ++i) {
    int rc = momms_gemm_validate(&descs[i]);
    if (rc) return fail(rc, "problem %d: %s", i, momms_last_error());
    const momms_gemm_desc& d = descs[i];
    if (d.m == 0 || d.n == 0 || d.k == 0) continue;
    const momms_operand* ops[3] = {&d.a, &d.b, &d.c};
    for (int j = 0; j < 3; ++j)
      if (!packed_of(*ops[j]) && (ops[j]->mem == MOMMS_MEM_HOST || !on_device(ops[j]->ptr)))
        return fail(MOMMS_ERR_INVALID_ARG, "problem %d: plans take device operands only", i);
  }
  Plan* p = new Plan();
  p->device = ds->device;
  p->async = async;
  p->stream = async_stream;
  std::vector<std::pair<void*, std::pair<size_t, size_t>>> pending;  // (dst, (offset, bytes)) of async uploads

  std::vector<int> dlist, slist;
  for (int i = 0; i < count; ++i) {
    const momms_gemm_desc& d = descs[i];
    if (d.m == 0 || d.n == 0 || d.k == 0) continue;
    if (d.precision == MOMMS_PREC_PLAIN && d.dtype == MOMMS_DTYPE_F64) dlist.push_back(i);
    else if (d.precision == MOMMS_PREC_PLAIN) slist.push_back(i);
    else p->other.push_back(PlanProblem{d, d.slices});
  }

  // ---- f64 group ----
  if (!dlist.empty()) {
    using namespace dmma;
    struct Cost {
      int idx;
      double tile_cost;
      int tiles;
      int64_t kblocks;
    };
    std::vector<Cost> cs;
    for (int i : dlist) {
      const momms_gemm_desc& d = descs[i];
      const int tiles = (int)(ceil_div(d.m, BM) * ceil_div(d.n, BN));
      // live 8x8 blocks of an average tile, times k-blocks
      const double live = (double)std::min<int64_t>(d.m, BM) * std::min<int64_t>(d.n, BN) / 64.0;
      const int64_t kb = ceil_div(d.k, BK);
      cs.push_back(Cost{i, live * (double)kb, tiles, kb});
    }
    std::vector<grouped::DProblem> probs;
    std::vector<CUtensorMap> maps;
    std::vector<std::pair<double, int>> order;  // (unit cost, index into cs)
    std::vector<int> splits(cs.size());
    for (size_t j = 0; j < cs.size(); ++j) {
      const momms_gemm_desc& d = descs[cs[j].idx];
      // the same split count as a single launch of this shape: a problem's
      // result does not depend on the batch it is in
      splits[j] = splits_f64(d.m, d.n, d.k, ds->sm_count);
      order.push_back({cs[j].tile_cost / splits[j], (int)j});
    }
    std::sort(order.begin(), order.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    int64_t units = 0, parts = 0, ctrs = 0;
    for (auto& oc : order) {
      const Cost& c = cs[oc.second];
      const momms_gemm_desc& d = descs[c.idx];
      grouped::DProblem P;
      memset(&P, 0, sizeof(P));
      P.m = d.m; P.n = d.n; P.k = d.k;
      P.alpha = d.alpha; P.beta = d.beta;
      P.c = static_cast<double*>(d.c.ptr);
      P.rsc = d.c.rs; P.csc = d.c.cs;
      P.tiles_m = (int)ceil_div(d.m, BM);
      P.tiles_n = (int)ceil_div(d.n, BN);
      int s = splits[oc.second];
      P.kb_split = ceil_div(c.kblocks, s);
      s = (int)ceil_div(c.kblocks, P.kb_split);
      P.splits = s;
      P.unit_begin = units;
      units += (int64_t)c.tiles * s;
      if (s > 1) {
        P.part_offset = parts;
        P.counter_offset = ctrs;
        parts += (int64_t)c.tiles * s * BM * BN;
        ctrs += c.tiles;
      }
      // tensor maps in each operand's own orientation (repacked copies for
      // strides TMA cannot take, exactly as a single launch does)
      CUtensorMap ma, mb;
      const DevGemm gv = devgemm_of(d);  // packed operands: their column-major copies
      DevMat a = gv.a, b = gv.b;
      int oa = dmma_orient(a, d.m, d.k, true), ob = dmma_orient(b, d.k, d.n, false);
      if (oa == 2) {
        const int64_t ld = round_up(d.m, 2);
        void* dst = nullptr;
        int rc = plan_alloc(p, &dst, (size_t)ld * d.k * 8);
        if (rc) { plan_free(p); return rc; }
        p->repacks.push_back(Plan::Repack{a, d.m, d.k, dst, ld});
        a = DevMat{dst, 1, ld};
        oa = 0;
      }
      if (ob == 2) {
        const int64_t ld = round_up(d.k, 2);
        void* dst = nullptr;
        int rc = plan_alloc(p, &dst, (size_t)ld * d.n * 8);
        if (rc) { plan_free(p); return rc; }
        p->repacks.push_back(Plan::Repack{b, d.k, d.n, dst, ld});
        b = DevMat{dst, 1, ld};
        ob = 1;
      }
      const bool a_xc = (oa == 0), b_xc = (ob == 0);
      uint64_t dims[2], strides[1];
      uint32_t box[2];
      if (a_xc) {
        dims[0] = d.m; dims[1] = d.k; strides[0] = (uint64_t)(d.k == 1 ? round_up(d.m * 8, 16) : a.cs * 8);
        box[0] = 16; box[1] = BK;
      } else {
        dims[0] = d.k; dims[1] = d.m; strides[0] = (uint64_t)(d.m == 1 ? round_up(d.k * 8, 16) : a.rs * 8);
        box[0] = BK; box[1] = BM;
      }
      int rc = encode_tiled(&ma, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, a.ptr, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
      if (!rc) {
        if (b_xc) {
          dims[0] = d.n; dims[1] = d.k; strides[0] = (uint64_t)(d.k == 1 ? round_up(d.n * 8, 16) : b.rs * 8);
          box[0] = 16; box[1] = BK;
        } else {
          dims[0] = d.k; dims[1] = d.n; strides[0] = (uint64_t)(d.n == 1 ? round_up(d.k * 8, 16) : b.cs * 8);
          box[0] = BK; box[1] = BN;
        }
        rc = encode_tiled(&mb, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, b.ptr, dims, strides, box, CU_TENSOR_MAP_SWIZZLE_128B);
      }
      if (rc) {
        plan_free(p);
        return rc;
      }
      P.flags = (a_xc ? 1 : 0) | (b_xc ? 2 : 0);
      probs.push_back(P);
      maps.push_back(ma);
      maps.push_back(mb);
    }
    p->nd = (int)probs.size();
    p->d_units = units;
    void* buf;
    int rc = plan_alloc(p, &buf, probs.size() * sizeof(grouped::DProblem));
    if (!rc) { p->d_probs = static_cast<grouped::DProblem*>(buf); rc = plan_alloc(p, &buf, maps.size() * sizeof(CUtensorMap)); }
    if (!rc) { p->d_maps = static_cast<CUtensorMap*>(buf); rc = plan_alloc(p, &buf, (size_t)parts * 8); }
    if (!rc) { p->d_partials = static_cast<double*>(buf); rc = plan_alloc(p, &buf, (size_t)ctrs * 4); }
    if (!rc) { p->d_counters = static_cast<unsigned*>(buf); rc = plan_alloc(p, &buf, 2 * sizeof(unsigned long long)); }
    if (!rc) p->d_next = static_cast<unsigned long long*>(buf);
    if (rc) { plan_free(p); return rc; }
    size_t off = p->host_tables.size();
    rc = plan_upload(p, p->d_probs, probs.data(), probs.size() * sizeof(grouped::DProblem));
    if (!rc && async) pending.push_back({p->d_probs, {off, probs.size() * sizeof(grouped::DProblem)}});
    off = p->host_tables.size();
    if (!rc) rc = plan_upload(p, p->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap));
    if (!rc && async) pending.push_back({p->d_maps, {off, maps.size() * sizeof(CUtensorMap)}});
    if (!rc) rc = plan_zero(p, p->d_counters, (size_t)ctrs * 4);
    if (!rc) rc = plan_zero(p, p->d_next, 2 * sizeof(unsigned long long));
    if (rc) { plan_free(p); return rc; }
  }

  // ---- f32 groups: each problem's tile (tuning table or model) decides its group ----
  if (!slist.empty()) {
    using namespace ffma;
    std::vector<std::pair<double, grouped::SProblem>> items[2];
    for (int i : slist) {
      const momms_gemm_desc& d = descs[i];
      const DevGemm gv = devgemm_of(d);  // packed operands: their column-major copies
      const DevMat& va = gv.a;
      const DevMat& vb = gv.b;
      if (!((va.rs == 1 || va.cs == 1) && (vb.rs == 1 || vb.cs == 1))) {
        plan_free(p);
        return fail(MOMMS_ERR_INVALID_ARG, "problem %d: grouped f32 operands need unit stride along one index", i);
      }
      grouped::SProblem P;
      memset(&P, 0, sizeof(P));
      const bool a_xc = (va.rs == 1) && !(va.cs == 1 && d.m == 1);
      const bool b_xc = (vb.cs == 1) && !(vb.rs == 1 && d.n == 1);
      const int64_t a_ld = a_xc ? va.cs : va.rs, b_ld = b_xc ? vb.rs : vb.cs;
      const bool vec = ((reinterpret_cast<uintptr_t>(va.ptr) | reinterpret_cast<uintptr_t>(vb.ptr)) & 15) == 0 &&
                       a_ld % 4 == 0 && b_ld % 4 == 0;
      P.o = Operands{static_cast<const float*>(va.ptr), va.rs, va.cs, static_cast<const float*>(vb.ptr), vb.rs,
                     vb.cs, d.m, d.n, d.k, a_xc, b_xc, vec};
      P.e = Epi{d.m, d.n, (float)d.alpha, (float)d.beta, static_cast<float*>(d.c.ptr), d.c.rs, d.c.cs};
      const PlainCfg cfg = plain_cfg(MOMMS_DTYPE_F32, d.m, d.n, d.k, ds->sm_count);
      const int TMv = cfg.tile == 1 ? 64 : 128;
      if (!offsets_fit_32(P.o)) p->sg[cfg.tile].wide = true;
      P.tiles_m = (int)ceil_div(d.m, TMv);
      P.tiles_n = (int)ceil_div(d.n, TMv);
      const int64_t kb = ceil_div(d.k, BK);
      const double tile_cost = (double)std::min<int64_t>(d.m, TMv) * std::min<int64_t>(d.n, TMv) * (double)kb;
      P.kb_split = ceil_div(kb, cfg.splits);
      P.splits = (int)ceil_div(kb, P.kb_split);
      items[cfg.tile].push_back({tile_cost / P.splits, P});
    }
    for (int t = 0; t < 2; ++t) {
      if (items[t].empty()) continue;
      const int TMv = t == 1 ? 64 : 128;
      Plan::SGroup& G = p->sg[t];
      std::sort(items[t].begin(), items[t].end(), [](const auto& a, const auto& b) { return a.first > b.first; });
      std::vector<grouped::SProblem> probs;
      int64_t units = 0, parts = 0, ctrs = 0;
      for (auto& it : items[t]) {
        grouped::SProblem P = it.second;
        const int64_t tiles = (int64_t)P.tiles_m * P.tiles_n;
        P.unit_begin = units;
        units += tiles * P.splits;
        if (P.splits > 1) {
          P.part_offset = parts;
          P.counter_offset = ctrs;
          parts += tiles * P.splits * TMv * TMv;
          ctrs += tiles;
        }
        probs.push_back(P);
      }
      G.ns = (int)probs.size();
      G.units = units;
      void* buf;
      int rc = plan_alloc(p, &buf, probs.size() * sizeof(grouped::SProblem));
      if (!rc) { G.probs = static_cast<grouped::SProblem*>(buf); rc = plan_alloc(p, &buf, (size_t)parts * 4); }
      if (!rc) { G.partials = static_cast<float*>(buf); rc = plan_alloc(p, &buf, (size_t)ctrs * 4 + 16); }
      if (!rc) { G.counters = static_cast<unsigned*>(buf); rc = plan_alloc(p, &buf, 2 * sizeof(unsigned long long)); }
      if (!rc) G.next = static_cast<unsigned long long*>(buf);
      if (rc) { plan_free(p); return rc; }
      const size_t off = p->host_tables.size();
      rc = plan_upload(p, G.probs, probs.data(), probs.size() * sizeof(grouped::SProblem));
      if (!rc && async) pending.push_back({G.probs, {off, probs.size() * sizeof(grouped::SProblem)}});
      if (!rc) rc = plan_zero(p, G.counters, (size_t)ctrs * 4 + 16);
      if (!rc) rc = plan_zero(p, G.next, 2 * sizeof(unsigned long long));
      if (rc) { plan_free(p); return rc; }
    }
  }

  // Ozaki problems with a data-chosen slice count: choose once now (one
  // sampled bound on the current operands), so that launches never wait.
  for (PlanProblem& pp : p->other) {
    if (pp.d.precision == MOMMS_PREC_OZAKI && pp.slices == 0) {
      int s = 0;
      int rc = ozaki_choose_slices(pp.d, &s, async ? async_stream : nullptr);
      if (rc) { plan_free(p); return rc; }
      pp.slices = s;
    }
  }
  // Emulated problems that qualify run together: their slice products in one
  // persistent launch (ozaki_batch_*); the rest keep their own sequences.
  {
    std::vector<DevGemm> gs;
    std::vector<int> sl;
    std::vector<PlanProblem> rest;
    for (PlanProblem& pp : p->other) {
      const DevGemm g = devgemm_of(pp.d);
      if (pp.d.precision == MOMMS_PREC_OZAKI && ozaki_batchable(g, pp.slices)) {
        gs.push_back(g);
        sl.push_back(pp.slices);
      } else {
        rest.push_back(pp);
      }
    }
    int clusters = 0;
    if (gs.size() >= 2 && sp_pairs_available(&clusters)) {
      const int rc = ozaki_batch_create(gs.data(), sl.data(), (int)gs.size(), async ? async_stream : nullptr, async,
                                        &p->ozb);
      if (rc) { plan_free(p); return rc; }
      p->other = rest;
    }
  }
  // stream-ordered uploads: the host copies live in p->host_tables (no more
  // appends from here on, so the addresses are stable)
  for (auto& pu : pending) {
    cudaError_t e = cudaMemcpyAsync(pu.first, p->host_tables.data() + pu.second.first, pu.second.second,
                                    cudaMemcpyHostToDevice, async_stream);
    if (e != cudaSuccess) {
      plan_free(p);
      return cuda_fail(e, "plan upload");
    }
  }
  *out = p;
  return MOMMS_OK;
}

void plan_destroy(Plan* p) { plan_free(p); }

int plan_launch(Plan* p, cudaStream_t s, int max_sms) {
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  if (ds->device != p->device) return fail(MOMMS_ERR_INVALID_ARG, "plan belongs to device %d", p->device);
  cudaError_t e;
  for (const Plan::Repack& r : p->repacks) {
    int rc = repack_colmajor(r.src, r.rows, r.cols, 8, r.dst, r.ld, s);
    if (rc) return rc;
  }
  if (p->nd) {
    const int sms = (max_sms > 0 && max_sms < ds->sm_count) ? max_sms : ds->sm_count;
    const int grid = (int)std::min<int64_t>(p->d_units, sms);
    KernelTimer kt(MOMMS_KERNEL_DGEMM_DMMA, s);
    grouped::dgemm_grouped_kernel<<<grid, dmma::THREADS, dmma::SMEM_BYTES, s>>>(
        p->d_maps, p->d_probs, p->nd, p->d_units, p->d_partials, p->d_counters, p->d_next, ds->status);
    note_launch();
    if ((e = launch_status()) != cudaSuccess) return cuda_fail(e, "grouped f64 launch");
  }
  for (int t = 0; t < 2; ++t) {
    const Plan::SGroup& G = p->sg[t];
    if (!G.ns) continue;
    const int sms = (max_sms > 0 && max_sms < ds->sm_count) ? max_sms : ds->sm_count;
    KernelTimer kt(MOMMS_KERNEL_SGEMM_FFMA, s);
    if (t == 1) {
      using T = ffma::Tile<64>;
      const int grid = (int)std::min<int64_t>(G.units, (int64_t)T::CTAS_PER_SM * sms);
      auto k = G.wide ? grouped::sgemm_grouped_kernel<64, uint64_t> : grouped::sgemm_grouped_kernel<64, uint32_t>;
      k<<<grid, T::THREADS, T::SMEM_BYTES, s>>>(G.probs, G.ns, G.units, G.next, G.partials, G.counters);
    } else {
      using T = ffma::Tile<128>;
      const int grid = (int)std::min<int64_t>(G.units, (int64_t)T::CTAS_PER_SM * sms);
      auto k = G.wide ? grouped::sgemm_grouped_kernel<128, uint64_t> : grouped::sgemm_grouped_kernel<128, uint32_t>;
      k<<<grid, T::THREADS, T::SMEM_BYTES, s>>>(G.probs, G.ns, G.units, G.next, G.partials, G.counters);
    }
    note_launch();
    if ((e = launch_status()) != cudaSuccess) return cuda_fail(e, "grouped f32 launch");
  }
  if (p->ozb) {
    const int rc = ozaki_batch_launch(p->ozb, s, max_sms);
    if (rc) return rc;
  }
  for (PlanProblem& pp : p->other) {
    const DevGemm g = devgemm_of(pp.d);
    int rc;
    if (pp.d.precision == MOMMS_PREC_OZAKI) {
      int used = 0;
      rc = launch_dgemm_ozaki(g, pp.d.target_rel_err, pp.slices, &used, s);
    } else {
      rc = launch_sgemm_tf32x3(g, s);
    }
    if (rc) return rc;
  }
  return MOMMS_OK;
}

}  // namespace momms

// ---------------------------------------------------------------------------
// extern "C"
// ---------------------------------------------------------------------------
extern "C" {

struct momms_plan_s {
  momms::Plan* p;
};

int momms_plan_create(const momms_gemm_desc* descs, int count, momms_plan* out) {
  if (!out) return momms::fail(MOMMS_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  momms::Plan* p = nullptr;
  int rc = momms::plan_create(descs, count, &p, nullptr, false);
  if (rc) return rc;
  *out = new momms_plan_s{p};
  return MOMMS_OK;
}

int momms_plan_launch(momms_plan plan, void* stream) {
  if (!plan) return momms::fail(MOMMS_ERR_INVALID_ARG, "plan is null");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (plan->p->graph) {
    cudaError_t e = cudaGraphLaunch(plan->p->graph, s);
    return e == cudaSuccess ? MOMMS_OK : momms::cuda_fail(e, "cudaGraphLaunch");
  }
  return momms::plan_launch(plan->p, s, 0);
}

int momms_plan_capture(momms_plan plan, void* stream) {
  if (!plan) return momms::fail(MOMMS_ERR_INVALID_ARG, "plan is null");
  momms::Plan* p = plan->p;
  if (p->graph) return MOMMS_OK;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return momms::cuda_fail(e, "capture stream");
  (void)stream;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(s);
    return momms::cuda_fail(e, "cudaStreamBeginCapture");
  }
  int rc = momms::plan_launch(p, s, 0);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(s, &g);
  cudaStreamDestroy(s);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return momms::cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&p->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    p->graph = nullptr;
    return momms::cuda_fail(e, "cudaGraphInstantiate");
  }
  return MOMMS_OK;
}

int momms_plan_destroy(momms_plan plan) {
  if (!plan) return MOMMS_OK;
  momms::plan_free(plan->p);
  delete plan;
  return MOMMS_OK;
}

int momms_gemm_grouped(const momms_gemm_desc* descs, int count, void* stream) {
  momms_plan plan = nullptr;
  int rc = momms_plan_create(descs, count, &plan);
  if (rc) return rc;
  rc = momms_plan_launch(plan, stream);
  cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (!rc && e != cudaSuccess) rc = momms::cuda_fail(e, "stream synchronize");
  momms_plan_destroy(plan);
  return rc;
}

}  // extern "C"
