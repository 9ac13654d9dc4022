// Out-of-core GEMM: a call with host operands that would not fit in the
// device-memory staging budget is computed in blocks of C (and slabs of k),
// with the operand blocks streamed through two device slots each.
//
// This is the reference's out-of-core / L4 blocking one level up the memory
// hierarchy: there, PartM / PartN of 23040 (src/exper/out_of_core.rs:77-87)
// or 3600 (src/exper/l4.rs:71-78) sit above the in-cache algorithm so that
// each block's working set stays in L3; here the blocks keep the working set
// inside the HBM budget while host DRAM holds the matrices. Streams:
//   copy-in (the device's copy stream)   H2D of the next blocks' operands
//   compute (the caller's stream)        one device GEMM per (i, j, p) block
//   copy-out (second copy stream)        D2H of each finished C block
// so that the transfers of block t+1 and the copy-back of block t-1 run
// while block t computes.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <vector>

#include "internal.h"

namespace momms {

namespace {

std::atomic<uint64_t> g_budget{0};  // 0 = automatic

constexpr size_t kSlack = 64ull << 20;  // allowance for small buffers and pool rounding
constexpr int64_t kGran = 256;         // block sizes are multiples of the 128 x 256 tiles
// Planning model: GB300's SM count, host<->device copy bandwidth with pinned
// memory (measured ~210 GB/s each way), and a per-launch overhead.
constexpr double kPlanSms = 152.0;
constexpr double kHostBw = 2.0e11;
constexpr double kLaunchS = 3e-5;

size_t esize(int dtype) { return dtype == MOMMS_DTYPE_F64 ? 8 : 4; }

// Device bytes of the staged copy of a rows x cols view (either orientation).
size_t slot_bytes(int64_t rows, int64_t cols, size_t es) {
  return (size_t)round_up(std::max<int64_t>(rows, 1), 16) * (size_t)round_up(std::max<int64_t>(cols, 1), 16) * es;
}

size_t block_footprint(const momms_gemm_desc& d, const bool host[3], int64_t mb, int64_t nb, int64_t kb) {
  const size_t es = esize(d.dtype);
  size_t bytes = work_bytes(d.dtype, d.precision, d.slices, mb, nb, kb) + kSlack;
  if (host[0]) bytes += 2 * slot_bytes(mb, kb, es);
  if (host[1]) bytes += 2 * slot_bytes(kb, nb, es);
  if (host[2]) bytes += 2 * slot_bytes(mb, nb, es);
  return bytes;
}

// Host <-> device bytes of a blocking (block counts bm x bn x bk).
double block_traffic(const momms_gemm_desc& d, const bool host[3], int64_t bm, int64_t bn, int64_t bk,
                     bool m_outer) {
  const double es = (double)esize(d.dtype);
  const double a = es * d.m * d.k, b = es * d.n * d.k, c = es * d.m * d.n;
  double t = 0.0;
  // With k whole, the operand indexed by the outer loop stays in its slot
  // while the inner loop runs; the inner one is reloaded per outer block
  // unless it is a single block.
  if (m_outer) {
    if (host[0]) t += (bk == 1) ? a : a * bn;
    if (host[1]) t += (bn == 1 && bk == 1) ? b : b * bm;
  } else {
    if (host[1]) t += (bk == 1) ? b : b * bm;
    if (host[0]) t += (bm == 1 && bk == 1) ? a : a * bn;
  }
  if (host[2]) t += (d.beta != 0.0 ? 2.0 : 1.0) * c;
  return t;
}

}  // namespace

size_t work_bytes(int dtype, int precision, int slices, int64_t m, int64_t n, int64_t k) {
  const double M = (double)m, N = (double)n, K = (double)k;
  double bytes;
  if (precision == MOMMS_PREC_OZAKI) {
    const int s = slices > 0 ? slices : 8;  // FP64-level targets take up to 8 slices
    // digit planes of A and B, one int32 sum plane per accumulation group
    // (tile-blocked: m and n padded to whole 128 x 256 tiles)
    const double groups = (double)ozaki_group_count(s, k);
    const double Mp = (double)round_up(m, 128), Np = (double)round_up(n, 256);
    bytes = 2.0 * s * (M + N) * (double)round_up(std::min<int64_t>(k, kOzakiMaxK), 8) + 4.0 * groups * Mp * Np +
            12.0 * (M + N);
  } else if (precision == MOMMS_PREC_SPLIT_TF32) {
    bytes = 8.0 * (M + N) * (double)round_up(k, 4);
  } else {
    (void)dtype;
    (void)K;
    bytes = 21.0 * 1024 * 1024;  // split-k partials: at most one 128 x 128 tile per SM
  }
  return (size_t)bytes;
}

size_t incore_bytes(const momms_gemm_desc& d, const bool host[3]) {
  const size_t es = esize(d.dtype);
  size_t bytes = work_bytes(d.dtype, d.precision, d.slices, d.m, d.n, d.k) + kSlack;
  if (host[0]) bytes += slot_bytes(d.m, d.k, es);
  if (host[1]) bytes += slot_bytes(d.k, d.n, es);
  if (host[2]) bytes += slot_bytes(d.m, d.n, es);
  return bytes;
}

uint64_t staging_budget() {
  const uint64_t b = g_budget.load();
  if (b) return b;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  // memory the library's pool holds but is not using is available too
  DeviceState* ds = device_state();
  if (ds && ds->pool) {
    uint64_t reserved = 0, used = 0;
    if (cudaMemPoolGetAttribute(ds->pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
        cudaMemPoolGetAttribute(ds->pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
      free_b += (size_t)(reserved - used);
    cudaGetLastError();
  }
  const uint64_t margin = std::max<uint64_t>(1ull << 30, total_b / 20);
  return free_b > margin ? free_b - margin : 0;
}

int plan_blocks(const momms_gemm_desc& d, const bool host[3], uint64_t budget, BlockPlan* out) {
  BlockPlan best;
  double best_cost = -1.0;
  // sustained rates of the device paths (FLOP/s) on a full GPU
  const double rate = d.precision == MOMMS_PREC_OZAKI        ? 3.9e13
                      : d.precision == MOMMS_PREC_SPLIT_TF32 ? 2.2e14
                      : d.dtype == MOMMS_DTYPE_F64           ? 1.05e12
                                                             : 4.4e13;
  auto blocks_of = [](int64_t x, int64_t count) {
    return std::min<int64_t>(x, round_up(ceil_div(x, count), kGran));
  };
  for (int64_t bk = 1; bk <= 64; ++bk) {
    const int64_t kb = blocks_of(d.k, bk);
    if (bk > 1 && blocks_of(d.k, bk - 1) == kb) continue;
    if (d.precision == MOMMS_PREC_OZAKI && kb > kOzakiMaxK) continue;
    for (int64_t bm = 1; bm <= 64; ++bm) {
      const int64_t mb = blocks_of(d.m, bm);
      if (bm > 1 && blocks_of(d.m, bm - 1) == mb) continue;
      for (int64_t bn = 1; bn <= 64; ++bn) {
        const int64_t nb = blocks_of(d.n, bn);
        if (bn > 1 && blocks_of(d.n, bn - 1) == nb) continue;
        const size_t fp = block_footprint(d, host, mb, nb, kb);
        if (fp > budget) continue;
        const int64_t cm = ceil_div(d.m, mb), cn = ceil_div(d.n, nb), ck = ceil_div(d.k, kb);
        // compute time: each block is one launch whose last wave of
        // 128 x 256 tiles may leave SMs idle
        const double tiles = (double)(ceil_div(mb, 128) * ceil_div(nb, 256));
        const double waves = std::ceil(tiles / kPlanSms);
        const double eff = tiles / (waves * kPlanSms);
        // per block: launch overhead, and for the tensor-core paths the
        // operand pre-pass (slicing / splitting ~9e10 elements/s; Ozaki adds
        // a bound sample and one host round trip)
        double per_block = kLaunchS;
        if (d.precision == MOMMS_PREC_OZAKI) per_block += 5e-4 + (double)(mb + nb) * (double)kb / 9e10;
        if (d.precision == MOMMS_PREC_SPLIT_TF32) per_block += (double)(mb + nb) * (double)kb / 9e10;
        const double t_comp =
            2.0 * (double)d.m * (double)d.n * (double)d.k / (rate * eff) + (double)(cm * cn * ck) * per_block;
        for (int mo = 0; mo < 2; ++mo) {
          const double traffic = block_traffic(d, host, cm, cn, ck, mo == 1);
          // transfers overlap the computation, except the first block's
          const double t_xfer = traffic / kHostBw;
          const double first = (double)block_footprint(d, host, mb, nb, kb) / 2.0 / kHostBw;
          // k slabs round C once per slab and redo each block's pre-pass:
          // taken only when they buy more than a quarter of the time
          const double cost = (std::max(t_comp, t_xfer) + first) * (ck > 1 ? 1.25 : 1.0);
          if (best_cost < 0.0 || cost < best_cost) {
            best_cost = cost;
            best.mb = mb;
            best.nb = nb;
            best.kb = kb;
            best.order_m_outer = (mo == 1);
            best.bytes = fp;
            best.host_traffic = traffic;
          }
        }
      }
    }
  }
  if (best_cost < 0.0)
    return fail(MOMMS_ERR_OUT_OF_MEMORY, "no blocking of the %lld x %lld x %lld problem fits the %llu-byte budget",
                (long long)d.m, (long long)d.n, (long long)d.k, (unsigned long long)budget);
  *out = best;
  return MOMMS_OK;
}

namespace {

// Two device slots for the blocks of one host operand.
struct Slots {
  bool used = false;
  void* buf[2] = {nullptr, nullptr};
  int64_t key[2] = {-1, -1};           // which block the slot holds
  cudaEvent_t loaded[2] = {nullptr, nullptr};  // its copy-in is done (copy-in stream)
  cudaEvent_t freed[2] = {nullptr, nullptr};   // its last reader / copy-out is done
  bool ever_freed[2] = {false, false};
  Staged st[2];
};

struct Task {
  int64_t ib, jb, pb;
};

}  // namespace

int gemm_streamed(const momms_gemm_desc& d, const bool host[3], const BlockPlan& plan, cudaStream_t s) {
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  if (!ds->copy_stream || !ds->copy_stream2) return fail(MOMMS_ERR_CUDA, "copy streams unavailable");
  const size_t es = esize(d.dtype);
  const int64_t mb = plan.mb, nb = plan.nb, kb = plan.kb;
  const int64_t cm = ceil_div(d.m, mb), cn = ceil_div(d.n, nb), ck = ceil_div(d.k, kb);
  cudaStream_t h2d = ds->copy_stream, d2h = ds->copy_stream2;
  const momms_operand* ops[3] = {&d.a, &d.b, &d.c};
  Slots slots[3];
  int rc = MOMMS_OK;
  int verdict = MOMMS_OK;  // MOMMS_ERR_TARGET_UNREACHABLE from any block
  cudaError_t e = cudaSuccess;
  cudaEvent_t ev_alloc = nullptr, ev_cols = nullptr, ev_end[2] = {nullptr, nullptr};

  auto mk = [&](cudaEvent_t* ev) {
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  };
  mk(&ev_alloc);
  mk(&ev_cols);
  mk(&ev_end[0]);
  mk(&ev_end[1]);
  const int64_t rows_max[3] = {mb, kb, mb}, cols_max[3] = {kb, nb, nb};
  for (int x = 0; x < 3 && e == cudaSuccess && !rc; ++x) {
    if (!host[x]) continue;
    Slots& sl = slots[x];
    sl.used = true;
    for (int q = 0; q < 2 && e == cudaSuccess; ++q) {
      e = scratch_alloc_raw(&sl.buf[q], slot_bytes(rows_max[x], cols_max[x], es), s);
      mk(&sl.loaded[q]);
      mk(&sl.freed[q]);
    }
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev_alloc, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(h2d, ev_alloc, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(d2h, ev_alloc, 0);
  if (e != cudaSuccess) rc = cuda_fail(e, "out-of-core set-up");

  // block (r0, c0, rows, cols) of operand x as a host view
  auto sub_op = [&](int x, int64_t r0, int64_t c0) {
    momms_operand o = *ops[x];
    o.ptr = static_cast<char*>(o.ptr) + (size_t)(r0 * o.rs + c0 * o.cs) * es;
    return o;
  };
  auto block_of = [&](int x, const Task& t, int64_t* r0, int64_t* c0, int64_t* rows, int64_t* cols) {
    const int64_t i0 = t.ib * mb, j0 = t.jb * nb, p0 = t.pb * kb;
    const int64_t mi = std::min(mb, d.m - i0), nj = std::min(nb, d.n - j0), kp = std::min(kb, d.k - p0);
    if (x == 0) { *r0 = i0; *c0 = p0; *rows = mi; *cols = kp; }
    else if (x == 1) { *r0 = p0; *c0 = j0; *rows = kp; *cols = nj; }
    else { *r0 = i0; *c0 = j0; *rows = mi; *cols = nj; }
  };
  auto key_of = [&](int x, const Task& t) -> int64_t {
    if (x == 0) return t.ib * ck + t.pb;
    if (x == 1) return t.pb * cn + t.jb;
    return t.ib * cn + t.jb;
  };
  auto slot_with = [&](int x, int64_t key) -> int {
    for (int q = 0; q < 2; ++q)
      if (slots[x].key[q] == key) return q;
    return -1;
  };

  std::vector<Task> tasks;
  tasks.reserve((size_t)(cm * cn * ck));
  if (plan.order_m_outer) {
    for (int64_t ib = 0; ib < cm; ++ib)
      for (int64_t jb = 0; jb < cn; ++jb)
        for (int64_t pb = 0; pb < ck; ++pb) tasks.push_back(Task{ib, jb, pb});
  } else {
    for (int64_t jb = 0; jb < cn; ++jb)
      for (int64_t ib = 0; ib < cm; ++ib)
        for (int64_t pb = 0; pb < ck; ++pb) tasks.push_back(Task{ib, jb, pb});
  }

  // Copy-in of task t's blocks into slots (the slot that task `keep` uses is
  // never evicted).
  auto issue_loads = [&](size_t t, const Task* keep) -> int {
    const Task& tk = tasks[t];
    for (int x = 0; x < 3; ++x) {
      if (!host[x]) continue;
      if (x == 2 && tk.pb != 0) continue;  // C is loaded once, before its first k slab
      const int64_t key = key_of(x, tk);
      if (slot_with(x, key) >= 0) continue;
      int q = 0;
      if (keep) {
        const int kq = slot_with(x, key_of(x, *keep));
        q = (kq == 0) ? 1 : 0;
      } else {
        q = (slots[x].key[0] < 0) ? 0 : 1;
      }
      Slots& sl = slots[x];
      cudaError_t ce = cudaSuccess;
      if (sl.ever_freed[q]) ce = cudaStreamWaitEvent(h2d, sl.freed[q], 0);
      if (ce != cudaSuccess) return cuda_fail(ce, "out-of-core copy-in");
      int64_t r0, c0, rows, cols;
      block_of(x, tk, &r0, &c0, &rows, &cols);
      const momms_operand o = sub_op(x, r0, c0);
      Staged& st = sl.st[q];
      st = Staged{};
      st.rows = rows;
      st.cols = cols;
      st.host = true;
      st.row_major = (o.cs == 1 && o.rs != 1);
      const int64_t inner = st.row_major ? cols : rows;
      st.ld = round_up(std::max<int64_t>(inner, 1), 16 / (int64_t)es);
      st.owned = sl.buf[q];
      st.dev = st.row_major ? DevMat{st.owned, st.ld, 1} : DevMat{st.owned, 1, st.ld};
      if (x < 2 || d.beta != 0.0) {
        int r = stage_copy_in(o, es, st, h2d);
        if (r) return r;
      }
      if ((ce = cudaEventRecord(sl.loaded[q], h2d)) != cudaSuccess) return cuda_fail(ce, "out-of-core copy-in");
      sl.key[q] = key;
    }
    return MOMMS_OK;
  };

  if (!rc && !tasks.empty()) rc = issue_loads(0, nullptr);
  for (size_t t = 0; t < tasks.size() && !rc; ++t) {
    const Task& tk = tasks[t];
    if (t + 1 < tasks.size()) {
      rc = issue_loads(t + 1, &tk);
      if (rc) break;
    }
    DevGemm g;
    g.dtype = d.dtype;
    int64_t r0, c0, rows, cols;
    block_of(2, tk, &r0, &c0, &rows, &cols);
    g.m = rows;
    g.n = cols;
    block_of(0, tk, &r0, &c0, &rows, &cols);
    g.k = cols;
    g.alpha = d.alpha;
    g.beta = (tk.pb == 0) ? d.beta : 1.0;  // later k slabs accumulate (src/composables/part.rs:96-110)
    DevMat* dm[3] = {&g.a, &g.b, &g.c};
    int q_used[3] = {-1, -1, -1};
    for (int x = 0; x < 3 && !rc; ++x) {
      if (host[x]) {
        const int q = slot_with(x, key_of(x, tk));
        if (q < 0) {
          rc = fail(MOMMS_ERR_CUDA, "out-of-core: block not staged");
          break;
        }
        q_used[x] = q;
        *dm[x] = slots[x].st[q].dev;
        if ((e = cudaStreamWaitEvent(s, slots[x].loaded[q], 0)) != cudaSuccess) rc = cuda_fail(e, "out-of-core wait");
      } else {
        block_of(x, tk, &r0, &c0, &rows, &cols);
        *dm[x] = DevMat{static_cast<char*>(ops[x]->ptr) + (size_t)(r0 * ops[x]->rs + c0 * ops[x]->cs) * es,
                        ops[x]->rs, ops[x]->cs};
      }
    }
    if (rc) break;
    momms_gemm_desc bd = d;
    bd.m = g.m;
    bd.n = g.n;
    bd.k = g.k;
    bd.beta = g.beta;
    rc = run_device_gemm(g, bd, s);
    if (rc == MOMMS_ERR_TARGET_UNREACHABLE) {  // the block holds a result; report after the rest
      verdict = rc;
      rc = MOMMS_OK;
    }
    if (rc) break;
    for (int x = 0; x < 2; ++x)
      if (host[x]) {
        Slots& sl = slots[x];
        if ((e = cudaEventRecord(sl.freed[q_used[x]], s)) != cudaSuccess) rc = cuda_fail(e, "out-of-core");
        sl.ever_freed[q_used[x]] = true;
      }
    if (!rc && host[2] && tk.pb == ck - 1) {
      // C block final: copy it back on the copy-out stream
      Slots& sl = slots[2];
      const int q = q_used[2];
      block_of(2, tk, &r0, &c0, &rows, &cols);
      const momms_operand o = sub_op(2, r0, c0);
      e = cudaEventRecord(ev_cols, s);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(d2h, ev_cols, 0);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "out-of-core copy-out");
        break;
      }
      rc = plain_pitch(o, sl.st[q]) ? stage_out_cols(o, es, sl.st[q], 0, cols, d2h) : stage_out(o, es, sl.st[q], d2h);
      if (rc) break;
      if ((e = cudaEventRecord(sl.freed[q], d2h)) != cudaSuccess) rc = cuda_fail(e, "out-of-core copy-out");
      sl.ever_freed[q] = true;
      sl.key[q] = -1;  // a finished C block is never read again
    }
  }

  // the caller's stream waits for both copy streams, then the slots go
  cudaError_t e2 = cudaSuccess;
  if (ev_end[0] && ev_end[1]) {
    e2 = cudaEventRecord(ev_end[0], h2d);
    if (e2 == cudaSuccess) e2 = cudaEventRecord(ev_end[1], d2h);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, ev_end[0], 0);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, ev_end[1], 0);
  }
  for (int x = 0; x < 3; ++x)
    for (int q = 0; q < 2; ++q)
      if (slots[x].buf[q]) cudaFreeAsync(slots[x].buf[q], s);
  cudaError_t e3 = cudaStreamSynchronize(s);
  if (!rc && e2 != cudaSuccess) rc = cuda_fail(e2, "out-of-core completion");
  if (!rc && e3 != cudaSuccess) rc = cuda_fail(e3, "stream synchronize");
  for (int x = 0; x < 3; ++x)
    for (int q = 0; q < 2; ++q) {
      if (slots[x].loaded[q]) cudaEventDestroy(slots[x].loaded[q]);
      if (slots[x].freed[q]) cudaEventDestroy(slots[x].freed[q]);
    }
  for (cudaEvent_t ev : {ev_alloc, ev_cols, ev_end[0], ev_end[1]})
    if (ev) cudaEventDestroy(ev);
  return rc ? rc : verdict;
}

}  // namespace momms

// ---------------------------------------------------------------------------
extern "C" {

int momms_set_staging_budget(uint64_t bytes) {
  momms::g_budget.store(bytes);
  return MOMMS_OK;
}

uint64_t momms_staging_budget(void) { return momms::staging_budget(); }

int momms_stream_plan(const momms_gemm_desc* desc, uint64_t budget, int64_t* mb, int64_t* nb, int64_t* kb) {
  if (!desc || !mb || !nb || !kb) return momms::fail(MOMMS_ERR_INVALID_ARG, "null argument");
  const momms_operand* ops[3] = {&desc->a, &desc->b, &desc->c};
  bool host[3];
  for (int i = 0; i < 3; ++i) host[i] = ops[i]->mem != MOMMS_MEM_DEVICE;  // AUTO counts as host here
  if (budget == 0) budget = momms::staging_budget();
  if (momms::incore_bytes(*desc, host) <= budget) {
    *mb = desc->m;
    *nb = desc->n;
    *kb = desc->k;
    return MOMMS_OK;
  }
  momms::BlockPlan p;
  int rc = momms::plan_blocks(*desc, host, budget, &p);
  if (rc) return rc;
  *mb = p.mb;
  *nb = p.nb;
  *kb = p.kb;
  return MOMMS_OK;
}

}  // extern "C"
