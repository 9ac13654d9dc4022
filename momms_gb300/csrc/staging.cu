// Host <-> device staging of operand views for calls with host operands.
#include <string.h>

#include <algorithm>
#include <vector>

#include "internal.h"

namespace momms {

bool is_device_ptr(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Device buffer for a rows x cols host view (column-major unless the view is
// row-major), allocated in stream order on `s`.
int stage_alloc(const momms_operand& op, int64_t rows, int64_t cols, size_t es, Staged& st, cudaStream_t s) {
  st.rows = rows;
  st.cols = cols;
  st.host = true;
  st.row_major = (op.cs == 1 && op.rs != 1);
  const int64_t inner = st.row_major ? cols : rows, outer = st.row_major ? rows : cols;
  st.ld = round_up(std::max<int64_t>(inner, 1), 16 / (int64_t)es);
  cudaError_t e = scratch_alloc(&st.owned, (size_t)st.ld * std::max<int64_t>(outer, 1) * es, s);
  if (e != cudaSuccess) return cuda_fail(e, "staging buffer");
  st.dev = st.row_major ? DevMat{st.owned, st.ld, 1} : DevMat{st.owned, 1, st.ld};
  return MOMMS_OK;
}

// A host view whose unit stride runs along the staged buffer's inner index
// and whose other stride leaves room for it: copied with one 2-D memcpy.
bool plain_pitch(const momms_operand& op, const Staged& st) {
  const int64_t inner = st.row_major ? st.cols : st.rows, outer = st.row_major ? st.rows : st.cols;
  const int64_t in_stride = st.row_major ? op.cs : op.rs, out_stride = st.row_major ? op.rs : op.cs;
  return in_stride == 1 && (outer == 1 || out_stride >= inner);
}

// Host -> device copy of the view into its staging buffer, on stream `s`.
int stage_copy_in(const momms_operand& op, size_t es, const Staged& st, cudaStream_t s) {
  const int64_t rows = st.rows, cols = st.cols;
  if (rows == 0 || cols == 0) return MOMMS_OK;
  const int64_t inner = st.row_major ? cols : rows, outer = st.row_major ? rows : cols;
  cudaError_t e;
  if (plain_pitch(op, st)) {
    const int64_t src_outer_stride = st.row_major ? op.rs : op.cs;
    const size_t spitch = (size_t)(outer == 1 ? inner : src_outer_stride) * es;
    e = cudaMemcpy2DAsync(st.owned, (size_t)st.ld * es, op.ptr, spitch, (size_t)inner * es, (size_t)outer,
                          cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "H2D copy");
    return MOMMS_OK;
  }
  // general strides: gather on the host, then one copy
  std::vector<char> tmp((size_t)st.ld * outer * es);
  for (int64_t j = 0; j < outer; ++j)
    for (int64_t i = 0; i < inner; ++i) {
      const int64_t r = st.row_major ? j : i, c = st.row_major ? i : j;
      memcpy(&tmp[((size_t)j * st.ld + i) * es], static_cast<const char*>(op.ptr) + (size_t)(r * op.rs + c * op.cs) * es,
             es);
    }
  e = cudaMemcpyAsync(st.owned, tmp.data(), tmp.size(), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "H2D copy");
  // the vector must outlive the copy
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "H2D copy");
  return MOMMS_OK;
}

// Host -> device copy of columns [j0, j1) of a plain-pitch view into its
// staging buffer, on stream `s` (the mirror of stage_out_cols).
int stage_in_cols(const momms_operand& op, size_t es, const Staged& st, int64_t j0, int64_t j1, cudaStream_t s) {
  if (st.rows == 0 || j1 <= j0) return MOMMS_OK;
  cudaError_t e;
  if (st.row_major) {  // each row holds columns j0..j1 contiguously
    e = cudaMemcpy2DAsync(static_cast<char*>(st.owned) + (size_t)j0 * es, (size_t)st.ld * es,
                          static_cast<const char*>(op.ptr) + (size_t)j0 * es,
                          (size_t)(st.rows == 1 ? st.cols : op.rs) * es, (size_t)(j1 - j0) * es, (size_t)st.rows,
                          cudaMemcpyHostToDevice, s);
  } else {  // columns j0..j1, each contiguous
    e = cudaMemcpy2DAsync(static_cast<char*>(st.owned) + (size_t)j0 * st.ld * es, (size_t)st.ld * es,
                          static_cast<const char*>(op.ptr) + (size_t)j0 * op.cs * es,
                          (size_t)(st.cols == 1 ? st.rows : op.cs) * es, (size_t)st.rows * es, (size_t)(j1 - j0),
                          cudaMemcpyHostToDevice, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "H2D copy");
  return MOMMS_OK;
}

// Device -> host copy of columns [j0, j1) of a staged C whose host view has a
// plain pitch (plain_pitch), on stream `s`.
int stage_out_cols(const momms_operand& op, size_t es, const Staged& st, int64_t j0, int64_t j1, cudaStream_t s) {
  if (st.rows == 0 || j1 <= j0) return MOMMS_OK;
  cudaError_t e;
  if (st.row_major) {  // each row holds columns j0..j1 contiguously
    e = cudaMemcpy2DAsync(static_cast<char*>(op.ptr) + (size_t)j0 * es, (size_t)(st.rows == 1 ? st.cols : op.rs) * es,
                          static_cast<const char*>(st.owned) + (size_t)j0 * es, (size_t)st.ld * es,
                          (size_t)(j1 - j0) * es, (size_t)st.rows, cudaMemcpyDeviceToHost, s);
  } else {  // columns j0..j1, each contiguous
    e = cudaMemcpy2DAsync(static_cast<char*>(op.ptr) + (size_t)j0 * op.cs * es,
                          (size_t)(st.cols == 1 ? st.rows : op.cs) * es,
                          static_cast<const char*>(st.owned) + (size_t)j0 * st.ld * es, (size_t)st.ld * es,
                          (size_t)st.rows * es, (size_t)(j1 - j0), cudaMemcpyDeviceToHost, s);
  }
  if (e != cudaSuccess) return cuda_fail(e, "D2H copy");
  return MOMMS_OK;
}

int stage_out(const momms_operand& op, size_t es, const Staged& st, cudaStream_t s) {
  const int64_t inner = st.row_major ? st.cols : st.rows, outer = st.row_major ? st.rows : st.cols;
  if (st.rows == 0 || st.cols == 0) return MOMMS_OK;
  const int64_t dst_inner_stride = st.row_major ? op.cs : op.rs;
  const int64_t dst_outer_stride = st.row_major ? op.rs : op.cs;
  cudaError_t e;
  if (dst_inner_stride == 1 && (outer == 1 || dst_outer_stride >= inner)) {
    const size_t dpitch = (size_t)(outer == 1 ? inner : dst_outer_stride) * es;
    e = cudaMemcpy2DAsync(op.ptr, dpitch, st.owned, (size_t)st.ld * es, (size_t)inner * es, (size_t)outer,
                          cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e, "D2H copy");
    return MOMMS_OK;
  }
  std::vector<char> tmp((size_t)st.ld * outer * es);
  e = cudaMemcpyAsync(tmp.data(), st.owned, tmp.size(), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "D2H copy");
  for (int64_t j = 0; j < outer; ++j)
    for (int64_t i = 0; i < inner; ++i) {
      const int64_t r = st.row_major ? j : i, c = st.row_major ? i : j;
      memcpy(static_cast<char*>(op.ptr) + (size_t)(r * op.rs + c * op.cs) * es, &tmp[((size_t)j * st.ld + i) * es],
             es);
    }
  return MOMMS_OK;
}

}  // namespace momms
