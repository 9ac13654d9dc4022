// Host-side internals shared by the momms GB300 translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/momms_gpu.h"

namespace momms {

// Per-device state created on first use.
struct DeviceState {
  int device = -1;
  int sm_count = 0;
  unsigned* status = nullptr;  // device status word (see DEV_* bits)
  cudaMemPool_t pool = nullptr;  // the library's stream-ordered scratch pool
  cudaStream_t copy_stream = nullptr;   // host->device staging copies of momms_gemm calls
  cudaStream_t copy_stream2 = nullptr;  // device->host copies (streamed calls, C write-back)
  cudaStream_t aux = nullptr;           // second compute stream of column-chunked emulated calls
  cudaStream_t aux2 = nullptr;          // emulated calls: the guaranteed bound and, under it, recombinations
};

// Stream-ordered scratch allocation (free with cudaFreeAsync) from the
// library's own pool, which keeps freed memory reserved instead of returning
// it to the driver at every synchronisation (the default pool's behaviour,
// which made each large call re-map its scratch). Inside stream capture it
// falls back to cudaMallocAsync (graph memory nodes).
cudaError_t scratch_alloc_raw(void** ptr, size_t bytes, cudaStream_t s);
template <typename T>
inline cudaError_t scratch_alloc(T** ptr, size_t bytes, cudaStream_t s) {
  return scratch_alloc_raw(reinterpret_cast<void**>(ptr), bytes, s);
}

// Returns a stream-ordered scratch allocation to the pool, in order on `s`,
// when it goes out of scope: on every return path of a launcher.
struct ScratchGuard {
  void* p;
  cudaStream_t s;
  ScratchGuard(void* ptr, cudaStream_t st) : p(ptr), s(st) {}
  ~ScratchGuard() {
    if (p) cudaFreeAsync(p, s);
  }
  ScratchGuard(const ScratchGuard&) = delete;
  ScratchGuard& operator=(const ScratchGuard&) = delete;
};

// Returns the state of the calling thread's current device (initialising it
// on first use), or nullptr with the error recorded.
DeviceState* device_state();

// ---- Host-side fault injection (momms_fault_inject) ----
// fault_take(kind) is true, using up one pending fault, when the next
// operation of that kind is to fail. device_malloc is cudaMalloc with
// injected out-of-memory failures; launch_status is the check made after a
// kernel launch (cudaGetLastError) with injected CUDA errors.
bool fault_take(int kind);
cudaError_t device_malloc(void** ptr, size_t bytes);
cudaError_t launch_status();
// A launcher that declines to launch (arguments its kernel cannot take)
// records the error here; the next launch_status() on this thread returns it.
void refuse_launch(cudaError_t e);

// Record an error message for momms_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// cuTensorMapEncodeTiled through the runtime's driver entry point, so that the
// library does not link libcuda directly.
int encode_tiled(CUtensorMap* map, CUtensorMapDataType dtype, uint32_t rank, const void* gaddr,
                 const uint64_t* dims, const uint64_t* strides_bytes, const uint32_t* box,
                 CUtensorMapSwizzle swizzle);

// A device-resident operand as the kernels see it: element (i, j) is at
// ptr[i * rs + j * cs].
struct DevMat {
  void* ptr;
  int64_t rs, cs;
};

// A call whose operands are being staged from host memory: their
// host->device copies run on a separate copy stream, and each kernel sequence
// waits (on its own stream) only for the operand it is about to read. C's
// device->host copy can start per column range as soon as that range is final.
struct Staging {
  cudaEvent_t ready[3] = {nullptr, nullptr, nullptr};  // A, B, C copied in; null = already on the device
  // Enqueues the copy-back of C's columns [j0, j1), final in stream order on
  // `s`; null when C is device memory or needs a host-side scatter.
  int (*writeback)(Staging* st, int64_t j0, int64_t j1, cudaStream_t s) = nullptr;
  void* ctx = nullptr;
  int64_t written = 0;  // columns of C handed to writeback so far
  // Deferred operands (B, C): not copied in yet; the launcher enqueues their
  // column ranges with copy_cols in the order it will read them. `done`
  // (may be null) receives an event marking the copy, owned by the call.
  bool deferred[3] = {false, false, false};
  int (*copy_cols)(Staging* st, int which, int64_t j0, int64_t j1, cudaEvent_t* done) = nullptr;
};

// A packed operand (momms_pack): the device-resident form a kernel reads.
struct PackedOperand {
  uint32_t magic = 0;  // kPackMagic while alive
  int device = -1;
  int dtype = 0, precision = 0, role = 0;  // role 0 = A (rows m, cols k), 1 = B (rows k, cols n)
  int64_t rows = 0, cols = 0;
  void* mem = nullptr;  // the one allocation
  size_t bytes = 0;
  // plain: column-major copy, leading dimension ld
  void* data = nullptr;
  int64_t ld = 0;
  // Ozaki / split-TF32: planes [np][R][kp] (R = m for A, n for B; k contiguous)
  void* planes = nullptr;
  int np = 0;  // Ozaki: slices; split-TF32: 2
  int64_t kp = 0;
  int* exps = nullptr;  // Ozaki: per-row (A) / per-column (B) exponents
};
constexpr uint32_t kPackMagic = 0x4D504B31u;
// The pack behind an operand flagged MOMMS_MEM_PACKED (nullptr otherwise).
inline const PackedOperand* packed_of(const momms_operand& op) {
  return op.mem == MOMMS_MEM_PACKED ? static_cast<const PackedOperand*>(op.ptr) : nullptr;
}

// One GEMM with all operands on the device (or arriving there, see Staging).
struct DevGemm {
  int dtype;  // momms_dtype
  int64_t m, n, k;
  double alpha, beta;
  DevMat a, b, c;
  Staging* staging = nullptr;
  const PackedOperand* pk[2] = {nullptr, nullptr};  // packed A, B (their DevMat is the plain copy, if any)
};

// DevGemm of a descriptor whose operands are device views or packs.
DevGemm devgemm_of(const momms_gemm_desc& d);
bool pack_is_live(const PackedOperand* p);
// Checks a packed operand against its position (0 = A, 1 = B) in `d`.
int check_packed(const momms_gemm_desc& d, int which, const PackedOperand* p);

// Make `s` wait until operand `which` (0 = A, 1 = B, 2 = C) is on the device.
inline cudaError_t wait_operand(const DevGemm& g, int which, cudaStream_t s) {
  if (!g.staging || !g.staging->ready[which]) return cudaSuccess;
  return cudaStreamWaitEvent(s, g.staging->ready[which], 0);
}
inline cudaError_t wait_operands(const DevGemm& g, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = wait_operand(g, i, s);
  return e;
}
// Enqueue the copy of a deferred operand's columns [j0, j1) (nothing for an
// operand already on the device; *done is then null).
inline int copy_columns(const DevGemm& g, int which, int64_t j0, int64_t j1, cudaEvent_t* done) {
  if (done) *done = nullptr;
  if (!g.staging || !g.staging->deferred[which] || j1 <= j0) return 0;
  return g.staging->copy_cols(g.staging, which, j0, j1, done);
}
// C's columns [j0, j1) are final in stream order on `s`.
inline int columns_done(const DevGemm& g, int64_t j0, int64_t j1, cudaStream_t s) {
  if (!g.staging || !g.staging->writeback || j1 <= j0) return 0;
  int rc = g.staging->writeback(g.staging, j0, j1, s);
  if (!rc) g.staging->written = j1;
  return rc;
}

// ---- Staging of host operand views (staging.cu) ----
bool is_device_ptr(const void* p);
// The device copy of a host view: column-major unless the view is row-major,
// leading dimension rounded up to 16 bytes.
struct Staged {
  DevMat dev{};
  void* owned = nullptr;
  bool host = false;
  int64_t rows = 0, cols = 0;
  bool row_major = false;  // layout of the device copy
  int64_t ld = 0;
};
int stage_alloc(const momms_operand& op, int64_t rows, int64_t cols, size_t es, Staged& st, cudaStream_t s);
// The view's unit stride runs along the device copy's inner index with room
// for it: one 2-D memcpy each way (otherwise the host gathers / scatters).
bool plain_pitch(const momms_operand& op, const Staged& st);
// Host -> device copy of columns [j0, j1) of a plain-pitch view.
int stage_in_cols(const momms_operand& op, size_t es, const Staged& st, int64_t j0, int64_t j1, cudaStream_t s);
int stage_copy_in(const momms_operand& op, size_t es, const Staged& st, cudaStream_t s);
int stage_out_cols(const momms_operand& op, size_t es, const Staged& st, int64_t j0, int64_t j1, cudaStream_t s);
int stage_out(const momms_operand& op, size_t es, const Staged& st, cudaStream_t s);

// Runs one GEMM on device (or arriving, see Staging) operands with the
// precision mode of `d` (api.cu).
int run_device_gemm(const DevGemm& g, const momms_gemm_desc& d, cudaStream_t s);

// Device bytes a mode needs beyond the operands for an m x n x k problem
// (slice planes, group sums, split-k partials); an upper bound.
size_t work_bytes(int dtype, int precision, int slices, int64_t m, int64_t n, int64_t k);

// ---- Out-of-core blocking (outofcore.cu) ----
// Block sizes of a streamed call: C in mb x nb blocks, k in slabs of kb,
// `order_m_outer` = loop over row blocks outside column blocks.
struct BlockPlan {
  int64_t mb = 0, nb = 0, kb = 0;
  bool order_m_outer = false;
  size_t bytes = 0;           // device bytes the plan holds
  double host_traffic = 0.0;  // host<->device bytes it moves
};
int plan_blocks(const momms_gemm_desc& d, const bool host[3], uint64_t budget, BlockPlan* out);
// Device bytes an unblocked call holds: staged host operands + work space.
size_t incore_bytes(const momms_gemm_desc& d, const bool host[3]);
// The staging budget in effect (momms_set_staging_budget, or the device's
// free memory less a margin).
uint64_t staging_budget();
// C := beta*C + alpha*A*B with at least one host operand, streamed in blocks.
int gemm_streamed(const momms_gemm_desc& d, const bool host[3], const BlockPlan& plan, cudaStream_t s);

// Launchers for the plain paths (device operands; asynchronous on `s`).
int launch_dgemm_dmma(const DevGemm& g, cudaStream_t s);
int launch_sgemm_ffma(const DevGemm& g, cudaStream_t s);
int launch_sgemm_tf32x3(const DevGemm& g, cudaStream_t s);
// Longest k of one emulated launch (8-bit digits: 511 k-blocks of 64 keep a
// digit pair's int32 sum exact); longer k runs in slabs accumulated into C.
constexpr int64_t kOzakiMaxK = 32704;
// Most slices of an emulated call: 15 digits of 8 bits (120 bits). The digit
// extraction works in 128-bit integers and the top digit of an s-slice split
// needs 8 * (s - 1) + 9 bits, so 16 slices would not fit.
constexpr int kOzakiMaxSlices = 15;
// Ozaki FP64 emulation: target relative error (0 = FP64 level) and slice count
// (0 = chosen from the target). *slices_used receives the count actually used.
int launch_dgemm_ozaki(const DevGemm& g, double target_rel_err, int slices, int* slices_used, cudaStream_t s);
// Accumulation groups (int32 sum planes) of an ns-slice product with this k.
int ozaki_group_count(int ns, int64_t k);
// Exponents of the R rows of a view x (element (r, p) at x[r*sr + p*sp],
// p < K) into exps[R], using maxbits[R] as scratch; and the ns digit planes
// [ns][R][kp] of the view under those exponents.
int ozaki_operand_exponents(const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K,
                            unsigned long long* maxbits, int* exps, cudaStream_t s);
void ozaki_operand_planes(int ns, const double* x, int64_t sr, int64_t sp, int64_t R, int64_t K, void* planes,
                          int64_t kp, const int* exps, cudaStream_t s);
// The two TF32 planes [2][R][kp] of an f32 view.
void tf32_operand_planes(const float* x, int64_t sr, int64_t sp, int64_t R, int64_t K, float* planes, int64_t kp,
                         cudaStream_t s);

// Copy an operand into a column-major device scratch matrix with an even
// leading dimension (used when its strides or alignment do not suit TMA or
// vector loads). `dst` must hold rows * round_up(ld) elements.
int repack_colmajor(const DevMat& src, int64_t rows, int64_t cols, size_t elem, void* dst, int64_t ld,
                    cudaStream_t s);

// How the f64 kernels stage an operand: 0 = TMA with the non-k index
// contiguous, 1 = TMA with k contiguous, 2 = needs a column-major repack.
int dmma_orient(const DevMat& v, int64_t rows, int64_t cols, bool x_is_rows);

// Launch configuration of a plain f64 / f32 problem: the output tile
// (0 = the kernel's 128 x 128 tile, 1 = its small tile: FFMA 64 x 64) and the
// k-split count, from the tuning table (momms_autotune, keyed by shape
// bucket) or the model. Depends only on the shape and the SM count.
struct PlainCfg {
  int tile;
  int splits;
};
PlainCfg plain_cfg(int dtype, int64_t m, int64_t n, int64_t k, int sm_count);
int splits_f64(int64_t m, int64_t n, int64_t k, int sm_count);

// Emulated problems of a plan run together: each problem's preparation and
// recombination, and ONE persistent slice-kernel launch (CTA pairs) over all
// of their tiles, from a device table of their schedules and tensor maps.
// Buffers and tables are made once at creation (`async`: stream-ordered on
// `s`, which is synchronised once for the table uploads). A problem qualifies
// with a fixed slice count, unpacked operands and k within one launch.
struct OzakiBatch;
bool ozaki_batchable(const DevGemm& g, int slices);
// True when this device can run the CTA-pair slice kernel (*clusters: pairs at once).
bool sp_pairs_available(int* clusters);
int ozaki_batch_create(const DevGemm* gs, const int* slices, int count, cudaStream_t s, bool async, OzakiBatch** out);
int ozaki_batch_launch(OzakiBatch* b, cudaStream_t s, int max_sms);
void ozaki_batch_destroy(OzakiBatch* b);

// Ozaki: choose the slice count for `d` from its target with the guaranteed
// bound (synchronises `s`).
int ozaki_choose_slices(const momms_gemm_desc& d, int* slices, cudaStream_t s);

// One-time per-device set-up of kernel attributes (dynamic shared memory
// limits), run by device_state() so that no launch path needs it (launch
// paths must stay legal inside stream capture).
int set_attrs_dmma();
int set_attrs_grouped();
int set_attrs_tf32();
int set_attrs_ozaki();

// Execution plans (grouped.cu). With `async`, allocations, uploads and frees
// are stream-ordered on `stream` (no device-wide synchronisation); otherwise
// plan_create is synchronous.
struct Plan;
int plan_create(const momms_gemm_desc* descs, int count, Plan** out, cudaStream_t stream, bool async);
// max_sms > 0 caps the persistent grids, leaving SMs for concurrent work.
int plan_launch(Plan* p, cudaStream_t s, int max_sms);
void plan_destroy(Plan* p);

// Record of the calling thread's current / last momms_gemm call.
momms_call_info& call_info();

// Counts kernel launches made by this library (momms_launch_count()).
void note_launch(int n = 1);

// Brackets the launches made during its lifetime with CUDA events on `s`
// when momms_timing_enable(1) is in effect (see momms_timing_read).
class KernelTimer {
 public:
  KernelTimer(int cls, cudaStream_t s);
  ~KernelTimer();
  KernelTimer(const KernelTimer&) = delete;
  KernelTimer& operator=(const KernelTimer&) = delete;

 private:
  int cls_;
  cudaStream_t s_;
  cudaEvent_t a_, b_;
};

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

}  // namespace momms
