// Throughput probes that give the roofline denominators this library reports
// against: the FP64 tensor-core MMA (DMMA) and FP32 FFMA issue rates of the
// current device, measured with CUDA events over register-only loops (no
// memory traffic). GB300's FP64 pipe is shared by DMMA and DFMA; its measured
// rate, not a data-sheet figure, is the FP64 peak here.
#include <atomic>

#include "common.cuh"
#include "internal.h"

namespace momms {

namespace {
std::atomic<unsigned long long> g_launches{0};

constexpr int kAcc = 8;

__global__ void dmma_peak_loop(double* out, int iters) {
  double c[kAcc][2];
  const double a = 1.0 + threadIdx.x * 1e-9, b = 1.0 - threadIdx.x * 1e-9;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) c[j][0] = c[j][1] = 0.0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < kAcc; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[j][0]), "+d"(c[j][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// The legacy integer tensor path (mma.sync m16n8k32, s8 x s8 -> s32): the
// alternative an INT8 Ozaki scheme would run on, since tcgen05 has no integer
// kind on sm_103a. 2*16*8*32 operations per instruction.
__global__ void imma_peak_loop(int* out, int iters) {
  int c[kAcc][4];
  const uint32_t a0 = 0x01020304u + threadIdx.x, b0 = 0x05060708u ^ threadIdx.x;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) c[j][0] = c[j][1] = c[j][2] = c[j][3] = 0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < kAcc; ++j)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
          : "+r"(c[j][0]), "+r"(c[j][1]), "+r"(c[j][2]), "+r"(c[j][3])
          : "r"(a0), "r"(a0 + 1), "r"(a0 + 2), "r"(a0 + 3), "r"(b0), "r"(b0 + 1));
  }
  int s = 0;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) s += c[j][0] + c[j][1] + c[j][2] + c[j][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma_peak_loop(float* out, int iters) {
  float c[kAcc];
  const float a = 1.0f + threadIdx.x * 1e-7f, b = 0.9999f;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) c[j] = (float)j;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < kAcc; ++j) c[j] = fmaf(c[j], b, a);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < kAcc; ++j) s += c[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

}  // namespace momms

extern "C" {

unsigned long long momms_launch_count(void) { return momms::g_launches.load(); }

int momms_measure_peak(int kind, double* tflops) {
  using namespace momms;
  if (!tflops || kind < 0 || kind > 2) return fail(MOMMS_ERR_INVALID_ARG, "momms_measure_peak: bad argument");
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  const int blocks = ds->sm_count * 4, threads = 256;
  void* out = nullptr;
  cudaError_t e = device_malloc((void**)&out, (size_t)blocks * threads * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "peak probe buffer");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = kind == 0 ? 1500 : (kind == 1 ? 40000 : 20000);
  float best_ms = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    if (kind == 0) dmma_peak_loop<<<blocks, threads>>>(static_cast<double*>(out), iters);
    else if (kind == 1) ffma_peak_loop<<<blocks, threads>>>(static_cast<float*>(out), iters);
    else imma_peak_loop<<<blocks, threads>>>(static_cast<int*>(out), iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best_ms) best_ms = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "peak probe");
  const double warp_steps = (double)blocks * (threads / 32) * iters * kAcc;
  const double flops = kind == 0   ? warp_steps * 512.0
                       : kind == 1 ? (double)blocks * threads * iters * kAcc * 2.0
                                   : warp_steps * 8192.0;
  *tflops = flops / (best_ms * 1e-3) / 1e12;
  return MOMMS_OK;
}

}  // extern "C"
