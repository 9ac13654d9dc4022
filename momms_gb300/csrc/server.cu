// GEMM serving loop: continuous batching of device-resident requests into
// grouped launches (momms_server_*).
//
// Clients submit requests whose operands already live in device memory. A
// request is admitted when its footprint (operands plus an estimate of the
// work space its mode needs) fits in the HBM budget next to the requests
// already admitted; larger-than-budget requests are refused at submission.
// One scheduler thread turns whatever has been admitted into a batch as soon
// as one of `max_inflight` streams is free, builds a stream-ordered plan
// (grouped.cu) and launches it, so requests that arrive while earlier batches
// run are admitted and started as slots and memory free up, and their work
// overlaps on the device. Every problem is planned from its own shape and
// data only, so a result is bit-identical alone and in any mix. Latency is
// measured on the host from submission to the moment the scheduler sees the
// batch's completion event. Each batch also carries two timing events on its
// stream, around its launch: their times relative to an event recorded when
// the server starts are the batch's device interval, reported per request, so
// that the overlap of batches on the GPU can be read off directly. NVTX
// ranges mark each batch's formation and launch on the scheduler thread and
// each completion (header-only NVTX v3: no cost unless a profiler attaches).
#include <nvtx3/nvToolsExt.h>
#include <stdio.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace momms {

namespace {

struct Request {
  momms_gemm_desc d;
  size_t footprint = 0;
  double flops = 0.0;
  double est_s = 0.0;
  double submit_s = 0.0, start_s = 0.0, done_s = 0.0;
  int status = MOMMS_OK;
  int batch_size = 0;
  bool done = false;
  uint64_t batch_id = 0;
  double dev_start_ms = -1.0, dev_end_ms = -1.0;  // the batch's device interval
};

struct Batch {
  std::vector<uint64_t> ids;
  Plan* plan = nullptr;
  cudaEvent_t ev_start = nullptr;  // before the launch, on the batch's stream
  cudaEvent_t ev = nullptr;        // after it: the batch is done when this completes
  int stream = 0;
  bool big = false;
  uint64_t id = 0;
};

// Requests estimated to run longer than this alone are "large".
constexpr double kQuantumS = 2e-3;

// Rough single-GPU time of a request: 2mnk over the mode's sustained rate.
double estimate_s(const momms_gemm_desc& d) {
  const double flops = 2.0 * (double)d.m * (double)d.n * (double)d.k;
  double rate = 1.0e12;                                        // plain f64 (DMMA)
  if (d.precision == MOMMS_PREC_OZAKI) rate = 2.0e13;          // emulated f64
  else if (d.precision == MOMMS_PREC_SPLIT_TF32) rate = 1.5e14;
  else if (d.dtype == MOMMS_DTYPE_F32) rate = 4.0e13;          // FFMA
  return flops / rate;
}

size_t footprint_of(const momms_gemm_desc& d) {
  const size_t es = d.dtype == MOMMS_DTYPE_F64 ? 8 : 4;
  const double m = (double)d.m, n = (double)d.n, k = (double)d.k;
  return (size_t)(es * (m * k + k * n + m * n)) + work_bytes(d.dtype, d.precision, d.slices, d.m, d.n, d.k);
}

}  // namespace

struct Server {
  momms_server_config cfg;
  int device = 0;
  std::vector<cudaStream_t> streams;
  std::vector<char> stream_busy;
  std::mutex mu;
  std::condition_variable cv_work;  // wakes the scheduler
  std::condition_variable cv_done;  // wakes waiters
  std::deque<uint64_t> pending;     // submitted, waiting for budget (FIFO)
  std::deque<uint64_t> ready;       // admitted, waiting for a stream
  std::unordered_map<uint64_t, Request> reqs;
  std::vector<Batch> inflight;
  size_t admitted_bytes = 0;
  uint64_t next_id = 1;
  bool stop = false;
  int launching = 0;  // batches taken from `ready` and not yet in `inflight`
  int big_inflight = 0;
  int sm_count = 0;
  cudaEvent_t ev0 = nullptr;  // the device clock's origin for batch intervals
  uint64_t next_batch = 1;

  bool idle() const { return pending.empty() && ready.empty() && inflight.empty() && launching == 0; }
  std::thread th;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  // statistics since the last reset
  std::vector<double> lat_ms;
  uint64_t submitted = 0, completed = 0, rejected = 0, failed = 0, batches = 0, batched = 0;
  double flops_done = 0.0, first_submit = -1.0, last_done = 0.0;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }

  void finish_request(uint64_t id, int status, int batch_size) {
    auto it = reqs.find(id);
    if (it == reqs.end()) return;
    Request& r = it->second;
    r.done = true;
    r.status = status;
    r.done_s = now();
    r.batch_size = batch_size;
    admitted_bytes -= r.footprint;
    completed += 1;
    if (status == MOMMS_OK) {
      flops_done += r.flops;
      lat_ms.push_back((r.done_s - r.submit_s) * 1e3);
    } else {
      failed += 1;
    }
    last_done = r.done_s;
  }

  void loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
      // 1. completed batches
      bool any_done = false;
      for (size_t i = 0; i < inflight.size();) {
        Batch& b = inflight[i];
        cudaError_t q = cudaEventQuery(b.ev);
        if (q == cudaErrorNotReady) {
          ++i;
          continue;
        }
        const int st = (q == cudaSuccess) ? MOMMS_OK : cuda_fail(q, "batch");
        float t_start = -1.0f, t_end = -1.0f;
        if (st == MOMMS_OK && (cudaEventElapsedTime(&t_start, ev0, b.ev_start) != cudaSuccess ||
                               cudaEventElapsedTime(&t_end, ev0, b.ev) != cudaSuccess)) {
          cudaGetLastError();
          t_start = t_end = -1.0f;
        }
        {
          char msg[96];
          snprintf(msg, sizeof(msg), "momms batch %llu done (%zu requests)", (unsigned long long)b.id, b.ids.size());
          nvtxMarkA(msg);
        }
        for (uint64_t id : b.ids) {
          Request& r = reqs[id];
          r.batch_id = b.id;
          r.dev_start_ms = t_start;
          r.dev_end_ms = t_end;
          finish_request(id, st, (int)b.ids.size());
        }
        plan_destroy(b.plan);
        cudaEventDestroy(b.ev_start);
        cudaEventDestroy(b.ev);
        stream_busy[b.stream] = 0;
        if (b.big) big_inflight -= 1;
        inflight.erase(inflight.begin() + i);
        any_done = true;
      }
      if (any_done) cv_done.notify_all();
      // 2. admission in arrival order, bounded by the HBM budget
      while (!pending.empty()) {
        Request& r = reqs[pending.front()];
        if (admitted_bytes + r.footprint > cfg.hbm_budget_bytes) break;
        admitted_bytes += r.footprint;
        ready.push_back(pending.front());
        pending.pop_front();
      }
      // 3. launch admitted work on every free stream
      while (!ready.empty()) {
        int sidx = -1;
        for (size_t s = 0; s < streams.size(); ++s)
          if (!stream_busy[s]) {
            sidx = (int)s;
            break;
          }
        if (sidx < 0) break;
        // Batch formation. A request estimated above the quantum runs as a
        // batch of its own, on at most max_inflight-1 streams at a time and
        // with its persistent grid capped to 3/4 of the SMs, so smaller
        // requests keep flowing next to it; smaller requests are batched in
        // arrival order up to the quantum (they may pass a waiting large one).
        Batch b;
        b.stream = sidx;
        std::vector<momms_gemm_desc> descs;
        double est = 0.0;
        const bool big_slot = big_inflight < (int)streams.size() - 1 || streams.size() == 1;
        for (auto it = ready.begin(); it != ready.end() && (int)b.ids.size() < cfg.max_batch;) {
          Request& r = reqs[*it];
          if (r.est_s > kQuantumS) {
            if (b.ids.empty() && big_slot) {
              b.big = true;
              b.ids.push_back(*it);
              descs.push_back(r.d);
              r.start_s = now();
              ready.erase(it);
              break;
            }
            ++it;
            continue;
          }
          if (!b.ids.empty() && est + r.est_s > kQuantumS) break;
          est += r.est_s;
          b.ids.push_back(*it);
          descs.push_back(r.d);
          r.start_s = now();
          it = ready.erase(it);
        }
        if (b.ids.empty()) break;
        if (b.big) big_inflight += 1;
        const int max_sms = (b.big && streams.size() > 1) ? (sm_count * 3) / 4 : 0;
        stream_busy[sidx] = 1;
        launching += 1;  // in no queue while the lock is released
        lk.unlock();
        cudaStream_t s = streams[sidx];
        {
          char msg[96];
          snprintf(msg, sizeof(msg), "momms batch %llu: plan + launch (%zu requests, stream %d)",
                   (unsigned long long)next_batch, descs.size(), sidx);
          nvtxRangePushA(msg);
        }
        int rc = plan_create(descs.data(), (int)descs.size(), &b.plan, s, true);
        cudaError_t e = cudaSuccess;
        if (!rc) {
          e = cudaEventCreate(&b.ev_start);
          if (e == cudaSuccess) e = cudaEventCreate(&b.ev);
          if (e == cudaSuccess) e = cudaEventRecord(b.ev_start, s);
          if (e != cudaSuccess) rc = cuda_fail(e, "batch event");
        }
        if (!rc) rc = plan_launch(b.plan, s, max_sms);
        if (!rc && (e = cudaEventRecord(b.ev, s)) != cudaSuccess) rc = cuda_fail(e, "batch event");
        // A batch that failed after some of its work was enqueued is finished
        // only when that work is: its requests' outputs are not touched again
        // once they are reported.
        if (rc) cudaStreamSynchronize(s);
        nvtxRangePop();
        lk.lock();
        launching -= 1;
        if (rc) {
          if (b.plan) plan_destroy(b.plan);
          if (b.ev_start) cudaEventDestroy(b.ev_start);
          if (b.ev) cudaEventDestroy(b.ev);
          for (uint64_t id : b.ids) finish_request(id, rc, (int)b.ids.size());
          stream_busy[sidx] = 0;
          if (b.big) big_inflight -= 1;
          cv_done.notify_all();
        } else {
          b.id = next_batch++;
          batches += 1;
          batched += b.ids.size();
          inflight.push_back(std::move(b));
        }
      }
      if (stop && idle()) break;
      // 4. sleep: poll completions while work is on the GPU
      if (!inflight.empty()) cv_work.wait_for(lk, std::chrono::microseconds(50));
      else cv_work.wait_for(lk, std::chrono::milliseconds(20));
    }
  }
};

}  // namespace momms

extern "C" {

struct momms_server_s {
  momms::Server* s;
};

int momms_server_create(const momms_server_config* cfg, momms_server* out) {
  using namespace momms;
  if (!out) return fail(MOMMS_ERR_INVALID_ARG, "out is null");
  *out = nullptr;
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  Server* sv = new Server();
  momms_server_config c;
  memset(&c, 0, sizeof(c));
  if (cfg) c = *cfg;
  if (c.hbm_budget_bytes == 0) c.hbm_budget_bytes = 60ull << 30;
  if (c.max_batch <= 0) c.max_batch = 64;
  if (c.max_inflight <= 0) c.max_inflight = 3;
  if (c.queue_capacity <= 0) c.queue_capacity = 4096;
  sv->cfg = c;
  sv->device = ds->device;
  sv->sm_count = ds->sm_count;
  for (int i = 0; i < c.max_inflight; ++i) {
    cudaStream_t s;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      for (cudaStream_t t : sv->streams) cudaStreamDestroy(t);
      delete sv;
      return cuda_fail(e, "server stream");
    }
    sv->streams.push_back(s);
    sv->stream_busy.push_back(0);
  }
  cudaError_t e0 = cudaEventCreate(&sv->ev0);
  if (e0 == cudaSuccess) e0 = cudaEventRecord(sv->ev0, sv->streams[0]);
  if (e0 == cudaSuccess) e0 = cudaEventSynchronize(sv->ev0);
  if (e0 != cudaSuccess) {
    for (cudaStream_t t : sv->streams) cudaStreamDestroy(t);
    if (sv->ev0) cudaEventDestroy(sv->ev0);
    delete sv;
    return cuda_fail(e0, "server clock event");
  }
  sv->th = std::thread([sv] { sv->loop(); });
  *out = new momms_server_s{sv};
  return MOMMS_OK;
}

int momms_server_submit(momms_server server, const momms_gemm_desc* desc, uint64_t* id) {
  using namespace momms;
  if (!server || !desc || !id) return fail(MOMMS_ERR_INVALID_ARG, "null argument");
  Server* sv = server->s;
  int rc = momms_gemm_validate(desc);
  if (rc) return rc;
  const momms_operand* ops[3] = {&desc->a, &desc->b, &desc->c};
  if (desc->m > 0 && desc->n > 0 && desc->k > 0)
    for (const momms_operand* op : ops) {
      if (packed_of(*op)) continue;  // packs live in device memory
      cudaPointerAttributes at;
      if (op->mem == MOMMS_MEM_HOST || cudaPointerGetAttributes(&at, op->ptr) != cudaSuccess ||
          !(at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return fail(MOMMS_ERR_INVALID_ARG, "served requests keep their operands resident in device memory");
      }
    }
  const size_t fp = footprint_of(*desc);
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->stop) return fail(MOMMS_ERR_SHUTDOWN, "server is stopping");
  if (fp > sv->cfg.hbm_budget_bytes) {
    sv->rejected += 1;
    return fail(MOMMS_ERR_ADMISSION, "request needs %zu bytes; the HBM budget is %llu", fp,
                (unsigned long long)sv->cfg.hbm_budget_bytes);
  }
  if ((int)(sv->pending.size() + sv->ready.size()) >= sv->cfg.queue_capacity)
    return fail(MOMMS_ERR_BUSY, "queue full (%d requests)", sv->cfg.queue_capacity);
  const uint64_t rid = sv->next_id++;
  Request r;
  r.d = *desc;
  r.footprint = fp;
  r.flops = 2.0 * (double)desc->m * (double)desc->n * (double)desc->k;
  r.est_s = estimate_s(*desc);
  r.submit_s = sv->now();
  if (sv->first_submit < 0) sv->first_submit = r.submit_s;
  sv->submitted += 1;
  if (desc->m == 0 || desc->n == 0 || desc->k == 0) {
    r.done = true;
    r.done_s = r.submit_s;
    sv->reqs[rid] = r;
    sv->completed += 1;
  } else {
    sv->reqs[rid] = r;
    sv->pending.push_back(rid);
  }
  *id = rid;
  sv->cv_work.notify_one();
  return MOMMS_OK;
}

static void fill_info(const momms::Request& r, momms_request_info* info) {
  if (!info) return;
  info->submit_s = r.submit_s;
  info->start_s = r.start_s;
  info->done_s = r.done_s;
  info->status = r.status;
  info->batch_size = r.batch_size;
  info->batch_id = r.batch_id;
  info->device_start_ms = r.dev_start_ms;
  info->device_end_ms = r.dev_end_ms;
}

int momms_server_poll(momms_server server, uint64_t id, momms_request_info* info) {
  using namespace momms;
  if (!server) return fail(MOMMS_ERR_INVALID_ARG, "server is null");
  Server* sv = server->s;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return fail(MOMMS_ERR_INVALID_ARG, "unknown request %llu", (unsigned long long)id);
  if (!it->second.done) return MOMMS_ERR_BUSY;
  fill_info(it->second, info);
  const int st = it->second.status;
  sv->reqs.erase(it);
  return st;
}

int momms_server_wait(momms_server server, uint64_t id, double timeout_s, momms_request_info* info) {
  using namespace momms;
  if (!server) return fail(MOMMS_ERR_INVALID_ARG, "server is null");
  Server* sv = server->s;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return fail(MOMMS_ERR_INVALID_ARG, "unknown request %llu", (unsigned long long)id);
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::microseconds((int64_t)(std::max(0.0, timeout_s) * 1e6));
  while (!sv->reqs[id].done) {
    if (sv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !sv->reqs[id].done)
      return MOMMS_ERR_BUSY;
  }
  Request r = sv->reqs[id];
  sv->reqs.erase(id);
  fill_info(r, info);
  return r.status;
}

int momms_server_drain(momms_server server, double timeout_s) {
  using namespace momms;
  if (!server) return fail(MOMMS_ERR_INVALID_ARG, "server is null");
  Server* sv = server->s;
  std::unique_lock<std::mutex> lk(sv->mu);
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::microseconds((int64_t)(std::max(0.0, timeout_s) * 1e6));
  while (!sv->idle()) {
    if (sv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !sv->idle())
      return MOMMS_ERR_BUSY;
  }
  return MOMMS_OK;
}

int momms_server_stats(momms_server server, momms_server_report* out, int reset) {
  using namespace momms;
  if (!server || !out) return fail(MOMMS_ERR_INVALID_ARG, "null argument");
  Server* sv = server->s;
  std::lock_guard<std::mutex> lk(sv->mu);
  memset(out, 0, sizeof(*out));
  out->submitted = sv->submitted;
  out->completed = sv->completed;
  out->rejected = sv->rejected;
  out->failed = sv->failed;
  out->batches = sv->batches;
  out->mean_batch = sv->batches ? (double)sv->batched / sv->batches : 0.0;
  out->flops_completed = sv->flops_done;
  out->busy_s = (sv->first_submit >= 0 && sv->last_done > sv->first_submit) ? sv->last_done - sv->first_submit : 0.0;
  out->tflops = out->busy_s > 0 ? sv->flops_done / out->busy_s / 1e12 : 0.0;
  out->admitted_bytes = sv->admitted_bytes;
  std::vector<double> l = sv->lat_ms;
  if (!l.empty()) {
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) {
      const double pos = q * (double)(l.size() - 1);
      const size_t i = (size_t)pos;
      const double f = pos - (double)i;
      return i + 1 < l.size() ? l[i] * (1 - f) + l[i + 1] * f : l[i];
    };
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    double sum = 0.0;
    for (double x : l) sum += x;
    out->mean_ms = sum / (double)l.size();
    out->max_ms = l.back();
  }
  if (reset) {
    sv->lat_ms.clear();
    sv->submitted = sv->completed = sv->rejected = sv->failed = sv->batches = sv->batched = 0;
    sv->flops_done = 0.0;
    sv->first_submit = -1.0;
    sv->last_done = 0.0;
  }
  return MOMMS_OK;
}

int momms_server_destroy(momms_server server) {
  if (!server) return MOMMS_OK;
  momms::Server* sv = server->s;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
    sv->cv_work.notify_all();
  }
  if (sv->th.joinable()) sv->th.join();
  for (cudaStream_t s : sv->streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  if (sv->ev0) cudaEventDestroy(sv->ev0);
  delete sv;
  delete server;
  return MOMMS_OK;
}

}  // extern "C"
