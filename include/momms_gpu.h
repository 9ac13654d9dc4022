/*
 * momms_gpu.h - C ABI of the GB300 (sm_103a) blocked matrix multiply.
 *
 * One call computes C := beta*C + alpha*A*B for an m x k matrix A, a k x n
 * matrix B and an m x n matrix C, each given as a strided view: element (i, j)
 * of an operand lives at ptr[i*rs + j*cs] (counted in elements). Column-major
 * storage is rs = 1, cs = leading dimension; row-major is cs = 1.
 *
 * It replaces, as one node, the reference's composed subtree
 *     PartN -> PartK -> PackB -> PartM -> PackA -> ParallelN -> KernelNM -> microkernel
 * (src/exper/l3_packing.rs:58-66 of tlrmchlsmth/momms), whose only foreign
 * function boundary is the BLIS microkernel
 *     bli_dgemm_haswell_asm_6x8(k, *alpha, *a, *b, *beta, *c, rs_c, cs_c, *aux, *cntx)
 *     (ukernels/bli_gemm_haswell_asm_d6x8.c:666-676, bound in Rust at
 *      src/kern/ukernel_wrapper.rs:40-53 and :73-90).
 * The operand contract follows the reference's views: alpha is the product of
 * the A and B scalars and beta is the C scalar (src/kern/kernel_nm.rs:44-45);
 * a view's pointer is the buffer at the view offset (RoCM::get_buffer,
 * src/matrix/general_stride.rs:244-257) with the matrix's row and column
 * strides (:42-43).
 *
 * Errors are returned as momms_status codes (the reference panics instead,
 * e.g. src/kern/ukernel_wrapper.rs:23-28); momms_last_error() gives a message.
 * No entry point throws or aborts.
 *
 * Memory: an operand flagged MOMMS_MEM_HOST (or detected as host memory under
 * MOMMS_MEM_AUTO) is staged through device memory by the library and the call
 * returns after C has been copied back. When all operands are device memory
 * the call is asynchronous on `stream` (a cudaStream_t; NULL = legacy default
 * stream).
 */
#ifndef MOMMS_GPU_H
#define MOMMS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MOMMS_ABI_VERSION 2

typedef enum {
  MOMMS_OK = 0,
  MOMMS_ERR_INVALID_ARG = 1,    /* negative size, null pointer, bad enum */
  MOMMS_ERR_UNSUPPORTED = 2,    /* dtype / precision combination not provided */
  MOMMS_ERR_CUDA = 3,           /* a CUDA runtime call failed */
  MOMMS_ERR_NO_DEVICE = 4,      /* no usable CUDA device */
  MOMMS_ERR_OUT_OF_MEMORY = 5,  /* device allocation failed */
  MOMMS_ERR_DEVICE_TIMEOUT = 6, /* a kernel's bounded wait expired */
  MOMMS_ERR_ADMISSION = 7,      /* serving: request larger than the budget */
  MOMMS_ERR_BUSY = 8,           /* serving: queue full or not ready */
  MOMMS_ERR_SHUTDOWN = 9,       /* serving: server stopped */
  MOMMS_ERR_TARGET_UNREACHABLE = 10 /* OZAKI with an automatic slice count: 15 slices (the most) cannot
                                       guarantee the requested error for every entry; C holds the 15-slice
                                       result and momms_last_info's bound_rel_err the bound that holds */
} momms_status;

typedef enum { MOMMS_DTYPE_F64 = 0, MOMMS_DTYPE_F32 = 1 } momms_dtype;

/* How the products are formed.
 * PLAIN: f64 on FP64 tensor-core MMA (DMMA); f32 on register-blocked FFMA.
 * The other modes are added by later entries of this header. */
typedef enum {
  MOMMS_PREC_PLAIN = 0,
  MOMMS_PREC_OZAKI = 1,      /* f64 only: FP64 emulated from fp16 slices on tcgen05 */
  MOMMS_PREC_SPLIT_TF32 = 2  /* f32 only: 3-term split TF32 on tcgen05 */
} momms_precision;

typedef enum { MOMMS_MEM_AUTO = 0, MOMMS_MEM_HOST = 1, MOMMS_MEM_DEVICE = 2, MOMMS_MEM_PACKED = 3 } momms_memspace;

/* A strided matrix view: element (i, j) at ptr[i*rs + j*cs]. */
typedef struct {
  void* ptr;
  int64_t rs;
  int64_t cs;
  int32_t mem; /* momms_memspace */
  int32_t reserved;
} momms_operand;

/* One GEMM request: C := beta*C + alpha*A*B. */
typedef struct {
  int32_t dtype;     /* momms_dtype */
  int32_t precision; /* momms_precision */
  int64_t m, n, k;
  double alpha, beta; /* used in the operands' dtype */
  momms_operand a, b, c;
  double target_rel_err; /* OZAKI: requested max |dC_ij| / (|A||B|)_ij; 0 = FP64 level (2^-52) */
  int32_t slices;        /* OZAKI: slice count 1..15 (8 bits each), 0 = chosen from target_rel_err so
                            that a rigorous bound holds for every entry (see momms_last_info) */
  int32_t flags;         /* reserved, must be 0 */
} momms_gemm_desc;

/* The node entry point: the GPU replacement of the composed subtree above. */
int momms_gemm(const momms_gemm_desc* desc, void* stream);

/* Typed convenience forms with the argument meaning of the reference
 * microkernel (alpha and beta passed by pointer, C strides rs_c / cs_c),
 * extended by m, n and the A / B strides because the node also replaces the
 * packing layers. Memory space is detected per operand (MOMMS_MEM_AUTO). */
int momms_dgemm(int64_t m, int64_t n, int64_t k, const double* alpha, const double* a, int64_t rs_a, int64_t cs_a,
                const double* b, int64_t rs_b, int64_t cs_b, const double* beta, double* c, int64_t rs_c,
                int64_t cs_c, void* stream);
int momms_sgemm(int64_t m, int64_t n, int64_t k, const float* alpha, const float* a, int64_t rs_a, int64_t cs_a,
                const float* b, int64_t rs_b, int64_t cs_b, const float* beta, float* c, int64_t rs_c,
                int64_t cs_c, void* stream);

/* f64 GEMM that allocates no memory, for callers that cannot: an application
 * whose device memory is already owned by its own pool or framework (a
 * cudaMalloc from this library would fail or compete with it), or a
 * latency-critical loop that cannot afford cudaMalloc / cudaFree, their
 * implicit device-wide synchronisation or an out-of-memory failure midway.
 * No counterpart in the reference (its packing buffers are heap allocations,
 * src/composables/pack.rs:336-344).
 *
 * Same arguments, same kernel and same tile / split-k plan as momms_dgemm, but
 * all of A, B and C must already be device memory, and A and B must each have
 * unit stride along one index with the other stride a multiple of 2 elements
 * and a 16-byte aligned base (other layouts would need a repack copy). The
 * split-k scratch is one device-global array of MOMMS_NOALLOC_SCRATCH_BYTES
 * (160 partial tiles of 128 x 128 doubles plus 1024 tile counters) that every
 * GPU loading this library holds until the process exits; a problem whose
 * split-k plan needs more than that is rejected with MOMMS_ERR_INVALID_ARG.
 * All calls on a device share that array and it keeps the last call's
 * contents, so calls that overlap on the GPU (other streams, or other host
 * threads) race and must be serialised by the caller. The first call on each
 * device runs a one-time set-up with that device current (it looks up the
 * addresses of the array and of a status word); make that first call before
 * any stream capture. A kernel whose bounded wait expires stops early, leaving
 * C partly updated, and sets a bit in the no-alloc status word, a second
 * device-global word of the library: momms_noalloc_status reads it. The
 * operands must be memory of the current device. Asynchronous on `stream`. */
#define MOMMS_NOALLOC_SCRATCH_BYTES 20975616
int momms_dgemm_noalloc(int64_t m, int64_t n, int64_t k, const double* alpha, const double* a, int64_t rs_a,
                        int64_t cs_a, const double* b, int64_t rs_b, int64_t cs_b, const double* beta, double* c,
                        int64_t rs_c, int64_t cs_c, void* stream);
/* Reads and clears the current device's no-alloc status word (bits set by
 * momms_dgemm_noalloc kernels whose bounded waits expired). Returns MOMMS_OK or
 * MOMMS_ERR_DEVICE_TIMEOUT; *bits (if non-null) receives the raw word.
 * Synchronises the device; allocates nothing. No reference counterpart. */
int momms_noalloc_status(uint32_t* bits);

/* ---- Packed operands --------------------------------------------------------
 * An operand used by many calls (a weight matrix, a basis) can be packed once
 * into the form the kernels read, in device memory: for MOMMS_PREC_OZAKI its
 * row exponents and `slices` fp16 digit planes, for MOMMS_PREC_SPLIT_TF32 its
 * two TF32 planes, for MOMMS_PREC_PLAIN a column-major copy with a TMA-ready
 * leading dimension. A call then names it as an operand with
 * mem = MOMMS_MEM_PACKED, ptr = the momms_packed handle (rs, cs ignored), and
 * skips that operand's pre-pass; an emulated call with a packed operand uses
 * the pack's slice count (both packs must agree) and needs no host round
 * trip to choose one, so it can be captured in a CUDA graph. Results are
 * bit-identical to the unpacked call with the same slice count. The
 * reference's counterpart is its Hierarch matrix type (src/matrix/hierarch.rs:
 * 18-140), which stores an operand in the blocked layout the algorithm walks
 * so that no packing happens at run time.
 *
 * role: MOMMS_ROLE_A (rows x cols = m x k) or MOMMS_ROLE_B (k x n); the pack
 * fits only that position and those sizes. src: host or device view (AUTO /
 * HOST / DEVICE). slices: OZAKI only, 1..15 (0 = 7 slices of 8 bits, the
 * count the FP64-level target takes for operands without a wide exponent
 * spread). Emulated calls with k > 32704 cannot use packed operands (their k
 * slabs re-scale per slab).
 * Synchronous; the pack owns its device memory until momms_packed_destroy. */
typedef enum { MOMMS_ROLE_A = 0, MOMMS_ROLE_B = 1 } momms_role;
typedef struct momms_packed_s* momms_packed;
int momms_pack(int dtype, int precision, int role, int64_t rows, int64_t cols, const momms_operand* src, int slices,
               void* stream, momms_packed* out);
int momms_packed_destroy(momms_packed packed);
/* Device bytes the pack holds. */
uint64_t momms_packed_bytes(momms_packed packed);

/* ---- Out-of-core (host-resident) GEMMs -----------------------------------
 * A momms_gemm call with host operands whose staged copies plus work space
 * would exceed the staging budget is computed in blocks: C in mb x nb blocks,
 * k in slabs of kb (later slabs accumulate with beta = 1, as the reference's
 * PartK does), the operand blocks streamed through two device slots each
 * while the previous block computes and the one before is copied back. The
 * reference's counterpart is its out-of-core / L4 blocking of PartM / PartN
 * above the in-cache algorithm (src/exper/out_of_core.rs:77-87,
 * src/exper/l4.rs:71-78). Each block is an independent device GEMM: with an
 * automatic Ozaki slice count every block meets the target on its own; with
 * k in one slab and a fixed slice count the Ozaki result is bit-identical to
 * the unblocked call.
 *
 * Budget in bytes (0 = automatic: the device's free memory, plus what the
 * library's pool holds unused, less max(1 GiB, 5 %)). Process-wide. */
int momms_set_staging_budget(uint64_t bytes);
uint64_t momms_staging_budget(void);
/* The blocking a call would use under `budget` (0 = the budget in effect),
 * without running it; operands flagged MOMMS_MEM_AUTO count as host memory.
 * mb = m, nb = n, kb = k when the call fits unblocked. MOMMS_ERR_OUT_OF_MEMORY
 * if no blocking fits. */
int momms_stream_plan(const momms_gemm_desc* desc, uint64_t budget, int64_t* mb, int64_t* nb, int64_t* kb);

/* ---- Grouped launches and execution plans --------------------------------
 * Many independent GEMMs run as one persistent kernel per dtype: every plain
 * f64 problem's tiles (and k-splits) are work units of one DMMA kernel, every
 * plain f32 problem's of one FFMA kernel per output tile size; the slice
 * products of all emulated (Ozaki) problems with unpacked operands and k up to
 * 32704 are work units of one tcgen05 kernel (each problem's digit planes are
 * prepared and its recombination run by its own small kernels); split-TF32
 * and other emulated problems run their own kernel sequences. Each problem is planned from its own
 * shape only (tile, split-k: the tuning table or the model), so a problem
 * gives bit-identical results alone (momms_gemm) and in any batch. Plans take
 * device operands only. The reference runs one composed algorithm per call
 * (src/exper/l3.rs:46-93); it has no batched form. */
typedef struct momms_plan_s* momms_plan;

/* Builds the problem tables, tensor maps and split-k workspaces once
 * (synchronous). Operand pointers are captured: later launches read the
 * current contents of the same buffers. An Ozaki problem with slices == 0 has
 * its slice count chosen here from the operands' current contents. */
int momms_plan_create(const momms_gemm_desc* descs, int count, momms_plan* out);
/* Enqueues the plan on `stream` (its CUDA graph if captured). Asynchronous;
 * launches of one plan must not overlap each other on the GPU (they share
 * the plan's workspaces). */
int momms_plan_launch(momms_plan plan, void* stream);
/* Captures the plan's launches into a CUDA graph owned by the plan; later
 * momms_plan_launch calls launch the graph (one launch for the whole batch). */
int momms_plan_capture(momms_plan plan, void* stream);
int momms_plan_destroy(momms_plan plan);
/* Convenience: create, launch, synchronise `stream`, destroy. */
int momms_gemm_grouped(const momms_gemm_desc* descs, int count, void* stream);

/* ---- Serving ---------------------------------------------------------------
 * A request loop with continuous batching. Requests keep their operands
 * resident in device memory; a request is admitted when its footprint
 * (operands plus the work space its mode needs) fits in the HBM budget next to
 * the requests already admitted, and is refused at submission when it could
 * never fit. A scheduler thread launches whatever has been admitted as a
 * grouped plan on one of `max_inflight` streams as soon as one is free, so
 * requests arriving while others run start as slots and memory free up and
 * overlap on the device. Results are bit-identical to momms_gemm on the same
 * request (planning depends on a problem alone). No reference counterpart:
 * the reference is a library of composed algorithms without a serving layer. */
typedef struct momms_server_s* momms_server;
typedef struct {
  uint64_t hbm_budget_bytes; /* admission budget (0 = 60 GiB) */
  int32_t max_batch;         /* requests per launch (0 = 64) */
  int32_t max_inflight;      /* batches on the GPU at once (0 = 3); a request
                                estimated over 2 ms runs alone, on at most
                                max_inflight-1 streams, with its persistent
                                grid capped to 3/4 of the SMs */
  int32_t queue_capacity;    /* waiting requests before submit says BUSY (0 = 4096) */
  int32_t reserved;
} momms_server_config;
typedef struct {
  double submit_s, start_s, done_s; /* seconds on the server's clock */
  int32_t status;                   /* momms_status of the request */
  int32_t batch_size;               /* requests in the launch it ran in */
  uint64_t batch_id;                /* the launch it ran in (numbered from 1) */
  double device_start_ms;           /* that launch's device interval: CUDA events on its stream before and */
  double device_end_ms;             /* after it, in ms after the server started (-1 if it failed) */
} momms_request_info;
typedef struct {
  uint64_t submitted, completed, rejected, failed, batches;
  double mean_batch;
  double p50_ms, p99_ms, mean_ms, max_ms; /* submit-to-completion latency */
  double flops_completed;                 /* 2mnk over completed requests */
  double busy_s;                          /* first submission to last completion */
  double tflops;                          /* flops_completed / busy_s / 1e12 */
  uint64_t admitted_bytes;                /* footprint admitted right now */
} momms_server_report;
int momms_server_create(const momms_server_config* cfg, momms_server* out);
/* MOMMS_ERR_ADMISSION: larger than the budget; MOMMS_ERR_BUSY: queue full. */
int momms_server_submit(momms_server server, const momms_gemm_desc* desc, uint64_t* id);
/* Request status when done (and forgets the request); MOMMS_ERR_BUSY if not. */
int momms_server_poll(momms_server server, uint64_t id, momms_request_info* info);
int momms_server_wait(momms_server server, uint64_t id, double timeout_s, momms_request_info* info);
/* Waits until nothing is queued or running (MOMMS_ERR_BUSY on timeout). */
int momms_server_drain(momms_server server, double timeout_s);
int momms_server_stats(momms_server server, momms_server_report* out, int reset);
/* Finishes the queued work, then stops the scheduler. */
int momms_server_destroy(momms_server server);

/* ---- Autotuning -----------------------------------------------------------
 * The runtime analogue of the reference's compile-time block sizes
 * (typenum NC/KC/MC/MR/NR, src/exper/l3_packing.rs:58-66): times the launch
 * configurations of a plain problem on its device operands (writing only a
 * scratch C) — every output tile the dtype's kernel has (f32: 128 x 128 with
 * two CTAs per SM, or 64 x 64 with eight), each with the k-split counts that
 * keep two k-blocks per split — and records the fastest in a process-wide
 * table keyed by shape bucket (dtype, precision, ceil(log2) of m, n and k)
 * that momms_gemm and plans consult. A configuration never changes which
 * products are summed in which order inside a split, and a problem's entry
 * does not depend on its batch. Synchronous. */
typedef struct {
  int32_t splits;     /* chosen k-split count */
  int32_t candidates; /* configurations timed */
  float best_ms;      /* time of the chosen configuration */
  int32_t tile;       /* chosen output tile: 0 = 128 x 128, 1 = the small tile (f32: 64 x 64) */
} momms_tune_result;
int momms_autotune(const momms_gemm_desc* desc, momms_tune_result* out, void* stream);
/* Tunes every shape bucket of a batch once (the bucket's first plain problem
 * stands for it); *tuned (may be null) receives the number of buckets timed. */
int momms_autotune_batch(const momms_gemm_desc* descs, int count, void* stream, int* tuned);
/* Table as text, one "dtype precision m n k splits tile" line per entry
 * (m, n, k: the bucket's largest shape; on import any shape of the bucket,
 * and the tile field may be left out for 0). */
int momms_tune_export(char* buf, size_t cap, size_t* needed);
int momms_tune_import(const char* text);
int momms_tune_clear(void);

/* What the calling thread's last momms_gemm that wrote C did (MOMMS_OK, or
 * MOMMS_ERR_TARGET_UNREACHABLE with the 15-slice result). No reference
 * counterpart (the reference's blocking is fixed at compile time). */
typedef struct {
  int32_t precision;      /* momms_precision actually run */
  int32_t slices;         /* OZAKI: slice count used (chosen or given) */
  int32_t pairs;          /* OZAKI: slice products formed (tensor-core GEMMs) */
  int32_t groups;         /* OZAKI: accumulation groups */
  int32_t splits;         /* plain paths: k splits */
  int32_t slice_variant;  /* tensor-core paths: slice kernel variant run: 0 = one CTA per tile,
                             2 = CTA pairs with one cta_group::2 MMA (1 is unused) */
  double bound_rel_err;   /* OZAKI with an automatic slice count: a rigorous bound on
                             max_ij |dC_ij| / (|A||B|)_ij of the product, over every entry (-1 otherwise) */
} momms_call_info;
int momms_last_info(momms_call_info* out);

/* Checks a descriptor without touching the GPU: sizes, strides, enums.
 * Returns MOMMS_OK or MOMMS_ERR_INVALID_ARG / MOMMS_ERR_UNSUPPORTED. */
int momms_gemm_validate(const momms_gemm_desc* desc);

/* Reads and clears the current device's status word (bits set by kernels
 * whose bounded waits expired). Returns MOMMS_OK or MOMMS_ERR_DEVICE_TIMEOUT;
 * *bits (if non-null) receives the raw word. Synchronises the device. */
int momms_device_status(uint32_t* bits);

/* Self-test of the bounded-wait failure path: launches one small kernel on
 * `stream` that waits on a shared-memory barrier nothing arrives on, gives up
 * after `polls` polls (1..2^20; the GEMM kernels allow 2^24, about a second),
 * sets DEV_TIMEOUT_FULL (bit 0) in a status word and returns, so that the
 * next momms_device_status (word 0) or momms_noalloc_status (word 1) reports
 * MOMMS_ERR_DEVICE_TIMEOUT. The GPU context stays usable. No reference
 * counterpart (the reference panics on the host, src/kern/ukernel_wrapper.rs:
 * 23-28). */
int momms_selftest_wait_expiry(uint32_t polls, int word, void* stream);

/* Host-side fault injection for tests of the error paths: the library's next
 * `count` operations of one kind fail as the real failure would be reported.
 * MOMMS_FAULT_ALLOC: device allocations (scratch, staging buffers, packs,
 * plans, autotuning) return out-of-memory; MOMMS_FAULT_CUDA: the check after
 * a kernel launch reports a CUDA error (the launch itself has been made). The
 * entry point that meets the fault returns MOMMS_ERR_OUT_OF_MEMORY or
 * MOMMS_ERR_CUDA and releases what it holds, and later calls run normally.
 * Process-wide; count 0 clears. No GPU fault is involved: the failure is
 * reported, not caused. momms_fault_pending returns the faults of `kind` not
 * yet used (-1 for an unknown kind). No reference counterpart. */
typedef enum { MOMMS_FAULT_ALLOC = 0, MOMMS_FAULT_CUDA = 1 } momms_fault_kind;
int momms_fault_inject(int kind, int count);
int momms_fault_pending(int kind);

/* Static description of the error codes, and the last error message of the
 * calling thread (empty string if none). */
const char* momms_status_string(int status);
const char* momms_last_error(void);

/* ABI version of the loaded library (MOMMS_ABI_VERSION at build time). */
int momms_abi_version(void);

/* Number of kernels this library has launched in this process (all devices).
 * No reference counterpart: evidence for benchmarks of what ran on the GPU. */
unsigned long long momms_launch_count(void);

/* Per-kernel timing, off by default. While on, every launch of the library's
 * kernels is bracketed by CUDA events on its launching stream and the elapsed
 * time is accumulated per kernel class (no host synchronisation on the launch
 * path; momms_timing_read synchronises the recorded events). No reference
 * counterpart (the reference times whole runs, src/util.rs:87-92). */
typedef enum {
  MOMMS_KERNEL_DGEMM_DMMA = 0,   /* plain f64 */
  MOMMS_KERNEL_SGEMM_FFMA = 1,   /* plain f32 */
  MOMMS_KERNEL_SLICE_OZAKI = 2,  /* tcgen05 slice products, Ozaki f64 */
  MOMMS_KERNEL_SLICE_TF32 = 3,   /* tcgen05 slice products, split-TF32 f32 */
  MOMMS_KERNEL_PREP = 4,         /* exponent scan, slicing / splitting, repack */
  MOMMS_KERNEL_COMBINE = 5,      /* Ozaki FP64 recombination */
  MOMMS_KERNEL_BOUND = 6,        /* Ozaki: guaranteed error bound (bf16 magnitude product on tcgen05) */
  MOMMS_KERNEL_CLASSES = 7
} momms_kernel_class;
int momms_timing_enable(int on);
int momms_timing_read(int kernel_class, double* total_ms, unsigned long long* launches, int reset);

/* Measures the current device's peak issue rate in TFLOP/s (TOP/s for
 * kind 2) with a register-only loop: kind 0 = FP64 tensor-core MMA (DMMA
 * m8n8k4), kind 1 = FP32 FFMA, kind 2 = the legacy INT8 tensor path
 * (mma.sync m16n8k32 s8 -> s32, the alternative to fp16 digits on tcgen05). The roofline denominators of the f64 and f32 plain
 * paths. No reference counterpart (the reference only reports GFLOP/s,
 * src/util.rs:94-97). Synchronises the device. */
int momms_measure_peak(int kind, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* MOMMS_GPU_H */
