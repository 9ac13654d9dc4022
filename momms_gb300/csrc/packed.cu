// Packed operands: an operand converted once into the form the kernels read
// (column-major TMA-ready copy, Ozaki digit planes with their exponents, or
// split-TF32 planes), kept in device memory for many calls. The reference's
// counterpart is the Hierarch matrix (src/matrix/hierarch.rs:18-140): storage
// laid out in the blocking the algorithm walks, so no packing runs per call.
#include <string.h>

#include <algorithm>
#include <mutex>
#include <unordered_set>

#include "internal.h"

namespace momms {

namespace {
// Live packs: a handle is looked up here before it is dereferenced, so a
// destroyed or foreign pointer is refused instead of read.
std::mutex g_pack_mu;
std::unordered_set<const PackedOperand*> g_packs;
}  // namespace

bool pack_is_live(const PackedOperand* p) {
  std::lock_guard<std::mutex> lk(g_pack_mu);
  return p && g_packs.count(p) != 0;
}

int check_packed(const momms_gemm_desc& d, int which, const PackedOperand* p) {
  const char name = which == 0 ? 'A' : 'B';
  if (!pack_is_live(p)) return fail(MOMMS_ERR_INVALID_ARG, "%c is not a live packed operand", name);
  if (p->role != which) return fail(MOMMS_ERR_INVALID_ARG, "%c: the pack was made for the other operand", name);
  // a pack is memory of the device it was made on; the kernels (TMA loads
  // included) may read only the current device's memory
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(MOMMS_ERR_NO_DEVICE, "no current CUDA device");
  }
  if (p->device != dev)
    return fail(MOMMS_ERR_INVALID_ARG, "%c: the pack lives on device %d, the call runs on device %d", name, p->device,
                dev);
  const int64_t rows = which == 0 ? d.m : d.k, cols = which == 0 ? d.k : d.n;
  if (p->rows != rows || p->cols != cols)
    return fail(MOMMS_ERR_INVALID_ARG, "%c: pack is %lld x %lld, the call needs %lld x %lld", name,
                (long long)p->rows, (long long)p->cols, (long long)rows, (long long)cols);
  if (p->dtype != d.dtype || p->precision != d.precision)
    return fail(MOMMS_ERR_INVALID_ARG, "%c: pack has dtype %d / precision %d, the call %d / %d", name, p->dtype,
                p->precision, d.dtype, d.precision);
  return MOMMS_OK;
}

DevGemm devgemm_of(const momms_gemm_desc& d) {
  DevGemm g;
  g.dtype = d.dtype;
  g.m = d.m;
  g.n = d.n;
  g.k = d.k;
  g.alpha = d.alpha;
  g.beta = d.beta;
  const momms_operand* ops[2] = {&d.a, &d.b};
  DevMat* dm[2] = {&g.a, &g.b};
  for (int i = 0; i < 2; ++i) {
    const PackedOperand* p = packed_of(*ops[i]);
    g.pk[i] = p;
    if (p) *dm[i] = DevMat{p->data, 1, p->ld};  // plain packs: the column-major copy
    else *dm[i] = DevMat{ops[i]->ptr, ops[i]->rs, ops[i]->cs};
  }
  g.c = DevMat{d.c.ptr, d.c.rs, d.c.cs};
  return g;
}

}  // namespace momms

extern "C" {

int momms_pack(int dtype, int precision, int role, int64_t rows, int64_t cols, const momms_operand* src, int slices,
               void* stream, momms_packed* out) {
  using namespace momms;
  if (!out || !src) return fail(MOMMS_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  if (dtype != MOMMS_DTYPE_F64 && dtype != MOMMS_DTYPE_F32) return fail(MOMMS_ERR_INVALID_ARG, "unknown dtype %d", dtype);
  if (precision < MOMMS_PREC_PLAIN || precision > MOMMS_PREC_SPLIT_TF32)
    return fail(MOMMS_ERR_INVALID_ARG, "unknown precision %d", precision);
  if (precision == MOMMS_PREC_OZAKI && dtype != MOMMS_DTYPE_F64)
    return fail(MOMMS_ERR_UNSUPPORTED, "Ozaki emulation is an f64 mode");
  if (precision == MOMMS_PREC_SPLIT_TF32 && dtype != MOMMS_DTYPE_F32)
    return fail(MOMMS_ERR_UNSUPPORTED, "split-TF32 is an f32 mode");
  if (role != MOMMS_ROLE_A && role != MOMMS_ROLE_B) return fail(MOMMS_ERR_INVALID_ARG, "role must be A or B");
  if (rows <= 0 || cols <= 0 || rows > INT32_MAX || cols > INT32_MAX)
    return fail(MOMMS_ERR_INVALID_ARG, "pack of %lld x %lld", (long long)rows, (long long)cols);
  if (src->mem == MOMMS_MEM_PACKED) return fail(MOMMS_ERR_INVALID_ARG, "source is already packed");
  if (!src->ptr || src->rs < 0 || src->cs < 0) return fail(MOMMS_ERR_INVALID_ARG, "bad source view");
  if (precision == MOMMS_PREC_OZAKI && (slices < 0 || slices > kOzakiMaxSlices))
    return fail(MOMMS_ERR_INVALID_ARG, "slice count %d outside 0..16", slices);
  // k is the operand's inner dimension: A's columns, B's rows
  const int64_t K = role == MOMMS_ROLE_A ? cols : rows;
  const int64_t R = role == MOMMS_ROLE_A ? rows : cols;
  if (precision == MOMMS_PREC_OZAKI && K > kOzakiMaxK)
    return fail(MOMMS_ERR_UNSUPPORTED, "packed emulated operands need k <= %lld", (long long)kOzakiMaxK);
  DeviceState* ds = device_state();
  if (!ds) return MOMMS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t es = dtype == MOMMS_DTYPE_F64 ? 8 : 4;

  // the source on the device: staged if it is host memory
  Staged st;
  DevMat v{src->ptr, src->rs, src->cs};
  const bool host = src->mem == MOMMS_MEM_HOST || (src->mem == MOMMS_MEM_AUTO && !is_device_ptr(src->ptr));
  int rc = MOMMS_OK;
  if (host) {
    rc = stage_alloc(*src, rows, cols, es, st, s);
    if (!rc) rc = stage_copy_in(*src, es, st, s);
    if (rc) {
      if (st.owned) cudaFreeAsync(st.owned, s);
      return rc;
    }
    v = st.dev;
  }

  PackedOperand* p = new PackedOperand();
  p->device = ds->device;
  p->dtype = dtype;
  p->precision = precision;
  p->role = role;
  p->rows = rows;
  p->cols = cols;
  cudaError_t ce = cudaSuccess;
  if (precision == MOMMS_PREC_PLAIN) {
    p->ld = round_up(rows, 16 / (int64_t)es);
    p->bytes = (size_t)p->ld * (size_t)cols * es;
    ce = device_malloc((void**)&p->mem, p->bytes);
    if (ce == cudaSuccess) {
      p->data = p->mem;
      rc = repack_colmajor(v, rows, cols, es, p->data, p->ld, s);
    }
  } else if (precision == MOMMS_PREC_OZAKI) {
    p->np = slices > 0 ? slices : 7;  // 56 bits: FP64 level for most data
    p->kp = round_up(K, 8);
    const size_t plane_bytes = (size_t)p->np * (size_t)R * (size_t)p->kp * 2;
    const size_t exps_off = round_up((int64_t)plane_bytes, 256);
    p->bytes = exps_off + (size_t)round_up((int64_t)((size_t)R * sizeof(int)), 8) + (size_t)R * sizeof(unsigned long long);
    ce = device_malloc((void**)&p->mem, p->bytes);
    if (ce == cudaSuccess) {
      p->planes = p->mem;
      p->exps = reinterpret_cast<int*>(static_cast<char*>(p->mem) + exps_off);
      unsigned long long* maxbits = reinterpret_cast<unsigned long long*>(
          static_cast<char*>(p->mem) + exps_off + round_up((int64_t)((size_t)R * sizeof(int)), 8));
      // the operand as R x K: A itself, B transposed
      const int64_t sr = role == MOMMS_ROLE_A ? v.rs : v.cs, sp = role == MOMMS_ROLE_A ? v.cs : v.rs;
      rc = ozaki_operand_exponents(static_cast<const double*>(v.ptr), sr, sp, R, K, maxbits, p->exps, s);
      if (!rc) ozaki_operand_planes(p->np, static_cast<const double*>(v.ptr), sr, sp, R, K, p->planes, p->kp, p->exps, s);
    }
  } else {  // split-TF32
    p->np = 2;
    p->kp = round_up(K, 4);
    p->bytes = 2 * (size_t)R * (size_t)p->kp * 4;
    ce = device_malloc((void**)&p->mem, p->bytes);
    if (ce == cudaSuccess) {
      p->planes = p->mem;
      const int64_t sr = role == MOMMS_ROLE_A ? v.rs : v.cs, sp = role == MOMMS_ROLE_A ? v.cs : v.rs;
      tf32_operand_planes(static_cast<const float*>(v.ptr), sr, sp, R, K, static_cast<float*>(p->planes), p->kp, s);
    }
  }
  if (ce == cudaSuccess) ce = launch_status();
  if (st.owned) cudaFreeAsync(st.owned, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (!rc && ce != cudaSuccess) rc = cuda_fail(ce, "pack");
  if (!rc && e2 != cudaSuccess) rc = cuda_fail(e2, "pack");
  if (rc) {
    if (p->mem) cudaFree(p->mem);
    delete p;
    return rc;
  }
  p->magic = kPackMagic;
  {
    std::lock_guard<std::mutex> lk(g_pack_mu);
    g_packs.insert(p);
  }
  *out = reinterpret_cast<momms_packed>(p);
  return MOMMS_OK;
}

int momms_packed_destroy(momms_packed packed) {
  using namespace momms;
  PackedOperand* p = reinterpret_cast<PackedOperand*>(packed);
  if (!p) return MOMMS_OK;
  {
    std::lock_guard<std::mutex> lk(g_pack_mu);
    if (!g_packs.erase(p)) return fail(MOMMS_ERR_INVALID_ARG, "not a live packed operand");
  }
  p->magic = 0;
  cudaError_t e = p->mem ? cudaFree(p->mem) : cudaSuccess;
  delete p;
  return e == cudaSuccess ? MOMMS_OK : cuda_fail(e, "pack free");
}

uint64_t momms_packed_bytes(momms_packed packed) {
  const momms::PackedOperand* p = reinterpret_cast<const momms::PackedOperand*>(packed);
  return momms::pack_is_live(p) ? (uint64_t)p->bytes : 0;
}

}  // extern "C"
