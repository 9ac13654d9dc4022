// Self-test of the device-side failure path: a kernel waits on an mbarrier
// that nothing arrives on, with a short poll limit, gives up, reports the
// expiry in a status word and returns. The context stays usable; the host
// reads the word with momms_device_status / momms_noalloc_status. This is the
// same bounded wait (mbar_wait_bounded) and the same report (report_status)
// that every pipeline wait of the GEMM kernels uses, with the limit lowered
// from about a second to what the caller passes.
#include "common.cuh"
#include "internal.h"

namespace momms {

unsigned* noalloc_status_word();  // dgemm_dmma.cu

namespace {

__global__ void wait_expiry_kernel(uint32_t polls, unsigned* status) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival completes phase 0; none comes
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!mbar_wait_bounded(&bar, 0, polls)) report_status(status, DEV_TIMEOUT_FULL);
  }
}

}  // namespace
}  // namespace momms

extern "C" int momms_selftest_wait_expiry(uint32_t polls, int word, void* stream) {
  using namespace momms;
  if (polls == 0 || polls > (1u << 20)) return fail(MOMMS_ERR_INVALID_ARG, "polls must be in 1..2^20");
  unsigned* target = nullptr;
  if (word == 0) {
    DeviceState* ds = device_state();
    if (!ds) return MOMMS_ERR_NO_DEVICE;
    target = ds->status;
  } else if (word == 1) {
    target = noalloc_status_word();
    if (!target) return MOMMS_ERR_CUDA;
  } else {
    return fail(MOMMS_ERR_INVALID_ARG, "word must be 0 (device status) or 1 (no-alloc status)");
  }
  wait_expiry_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(polls, target);
  note_launch();
  cudaError_t e = launch_status();
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "wait-expiry self-test launch");
}
