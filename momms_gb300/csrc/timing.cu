// Per-kernel timing with CUDA events on the launching stream
// (momms_timing_enable / momms_timing_read).
#include <mutex>
#include <vector>

#include "internal.h"

namespace momms {

namespace {
struct Pending {
  int cls;
  cudaEvent_t a, b;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
double g_total[MOMMS_KERNEL_CLASSES];
unsigned long long g_count[MOMMS_KERNEL_CLASSES];

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return e;
}

// Folds finished pairs into the totals (caller holds g_mu). With `wait`,
// blocks until every recorded pair has completed.
void collect(bool wait) {
  std::vector<Pending> keep;
  for (const Pending& p : g_pending) {
    if (wait) cudaEventSynchronize(p.b);
    if (cudaEventQuery(p.b) != cudaSuccess) {
      cudaGetLastError();
      keep.push_back(p);
      continue;
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g_total[p.cls] += ms;
      g_count[p.cls] += 1;
    } else {
      cudaGetLastError();
    }
    g_pool.push_back(p.a);
    g_pool.push_back(p.b);
  }
  g_pending.swap(keep);
}
}  // namespace

KernelTimer::KernelTimer(int cls, cudaStream_t s) : cls_(cls), s_(s), a_(nullptr), b_(nullptr) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_on) return;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return;
  }
  if (g_pending.size() > 4096) collect(false);
  a_ = take_event();
  b_ = take_event();
  if (!a_ || !b_) {
    a_ = b_ = nullptr;
    return;
  }
  cudaEventRecord(a_, s_);
}

KernelTimer::~KernelTimer() {
  if (!a_) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEventRecord(b_, s_);
  g_pending.push_back(Pending{cls_, a_, b_});
}

}  // namespace momms

extern "C" {

int momms_timing_enable(int on) {
  std::lock_guard<std::mutex> lk(momms::g_mu);
  momms::g_on = on != 0;
  return MOMMS_OK;
}

int momms_timing_read(int kernel_class, double* total_ms, unsigned long long* launches, int reset) {
  if (kernel_class < 0 || kernel_class >= MOMMS_KERNEL_CLASSES)
    return momms::fail(MOMMS_ERR_INVALID_ARG, "kernel class %d out of range", kernel_class);
  std::lock_guard<std::mutex> lk(momms::g_mu);
  momms::collect(true);
  if (total_ms) *total_ms = momms::g_total[kernel_class];
  if (launches) *launches = momms::g_count[kernel_class];
  if (reset) {
    momms::g_total[kernel_class] = 0.0;
    momms::g_count[kernel_class] = 0;
  }
  return MOMMS_OK;
}

}  // extern "C"
