// momms/gemm_node.hpp - the reference's GemmNode composition API in C++17,
// with a GPU leaf node.
//
// Mirrors tlrmchlsmth/momms: an algorithm is a nested type of nodes that each
// implement `run(a, b, c, thr)`, a default constructor and a static
// `hierarchy_description()` (src/composables/mod.rs:24-36). Matrices are
// strided views with stacks of (offset, padding, iter_size) per axis
// (src/matrix/general_stride.rs, src/matrix/view.rs). The GPU leaf `GpuGemm`
// replaces the reference's PackB/PartM/PackA/ParallelN/KernelNM subtree with
// one momms_gemm call, so composed algorithms keep working above it, e.g. the
// out-of-core blocking of src/exper/out_of_core.rs:77-87:
//
//   using Algo = momms::SpawnThreads<momms::PartM<14400, momms::PartN<14400, momms::GpuGemm<double>>>>;
//
// Errors from the library become std::runtime_error (the reference panics).
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../momms_gpu.h"

namespace momms {

// ---------------------------------------------------------------------------
// Algorithm description (src/composables/mod.rs:24-29)
// ---------------------------------------------------------------------------
enum class StepKind { M, N, K };
struct AlgorithmStep {
  StepKind kind;
  size_t bsz;
  bool operator==(const AlgorithmStep& o) const { return kind == o.kind && bsz == o.bsz; }
};

// ---------------------------------------------------------------------------
// Views (src/matrix/view.rs)
// ---------------------------------------------------------------------------
struct MatrixView {
  size_t offset = 0, padding = 0, iter_size = 0;
  size_t physical_size() const { return iter_size > padding ? iter_size - padding : 0; }
  // (iter size, padding) of the block of `blksz` starting at `index`
  std::pair<size_t, size_t> zoomed_size_and_padding(size_t index, size_t blksz) const {
    const size_t zs = std::min(blksz, iter_size - index);
    const size_t phys = physical_size();
    const std::ptrdiff_t pad = (std::ptrdiff_t)(index + zs) - (std::ptrdiff_t)std::max(index, phys);
    return {zs, pad > 0 ? (size_t)pad : 0};
  }
};

// ---------------------------------------------------------------------------
// Matrix<T>: a strided matrix with view stacks and a scalar
// (src/matrix/general_stride.rs). Column-major by default; transpose() swaps
// the strides. The buffer is host memory, 4096-byte aligned.
// ---------------------------------------------------------------------------
template <typename T>
class Matrix {
  static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value, "Matrix<T>: T is double or float");

 public:
  Matrix(size_t h, size_t w) : rs_(1), cs_(h), owner_(true) {
    const size_t bytes = std::max<size_t>(1, ((h * w * sizeof(T)) + 4095) / 4096 * 4096);
    buf_ = static_cast<T*>(std::aligned_alloc(4096, bytes));
    if (!buf_) throw std::bad_alloc();
    y_.push_back(MatrixView{0, 0, h});
    x_.push_back(MatrixView{0, 0, w});
  }
  // A view onto memory owned elsewhere (host or device), element (i, j) at
  // ptr[i*rs + j*cs].
  Matrix(T* ptr, size_t h, size_t w, size_t rs, size_t cs) : buf_(ptr), rs_(rs), cs_(cs), owner_(false) {
    y_.push_back(MatrixView{0, 0, h});
    x_.push_back(MatrixView{0, 0, w});
  }
  Matrix(const Matrix&) = delete;
  Matrix& operator=(const Matrix&) = delete;
  Matrix(Matrix&& o) noexcept { *this = std::move(o); }
  Matrix& operator=(Matrix&& o) noexcept {
    std::swap(buf_, o.buf_);
    rs_ = o.rs_;
    cs_ = o.cs_;
    alpha_ = o.alpha_;
    y_ = std::move(o.y_);
    x_ = std::move(o.x_);
    std::swap(owner_, o.owner_);
    return *this;
  }
  ~Matrix() {
    if (owner_) std::free(buf_);
  }

  // A non-owning copy of the current (top) views, as SpawnThreads hands to
  // each worker (general_stride.rs:196-211; here padding stays the view's own).
  Matrix alias() const {
    Matrix m(buf_, 0, 0, rs_, cs_);
    m.y_.assign(1, y_.back());
    m.x_.assign(1, x_.back());
    m.alpha_ = alpha_;
    return m;
  }

  size_t height() const { return y_.back().physical_size(); }
  size_t width() const { return x_.back().physical_size(); }
  size_t iter_height() const { return y_.back().iter_size; }
  size_t iter_width() const { return x_.back().iter_size; }
  size_t row_stride() const { return rs_; }
  size_t column_stride() const { return cs_; }
  T scalar() const { return alpha_; }
  void set_scalar(T a) { alpha_ = a; }

  // Pointer at the current view offset (RoCM::get_buffer, general_stride.rs:244-250).
  T* buffer() const { return buf_ + y_.back().offset * rs_ + x_.back().offset * cs_; }
  T get(size_t y, size_t x) const { return buffer()[y * rs_ + x * cs_]; }
  void set(size_t y, size_t x, T v) { buffer()[y * rs_ + x * cs_] = v; }

  void transpose() {
    if (y_.size() != 1 || x_.size() != 1) throw std::logic_error("can't transpose a submatrix");
    std::swap(y_, x_);
    std::swap(rs_, cs_);
  }

  size_t push_y_view(size_t blksz) { return push(y_, blksz); }
  size_t push_x_view(size_t blksz) { return push(x_, blksz); }
  void pop_y_view() { y_.pop_back(); }
  void pop_x_view() { x_.pop_back(); }
  void slide_y_view_to(size_t y, size_t blksz) { slide(y_, y, blksz); }
  void slide_x_view_to(size_t x, size_t blksz) { slide(x_, x, blksz); }
  void push_y_split(size_t start, size_t end) { split(y_, start, end, height()); }
  void push_x_split(size_t start, size_t end) { split(x_, start, end, width()); }
  void pop_y_split() { y_.pop_back(); }
  void pop_x_split() { x_.pop_back(); }

  // uniform [-1, 1) from a seeded generator (the reference's fill_rand,
  // src/matrix/matrix.rs:162-169, is unseeded)
  void fill_rand(uint64_t seed) {
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    for (size_t x = 0; x < width(); ++x)
      for (size_t y = 0; y < height(); ++y) set(y, x, (T)u(g));
  }
  void fill_zero() {
    for (size_t x = 0; x < width(); ++x)
      for (size_t y = 0; y < height(); ++y) set(y, x, T(0));
  }

 private:
  static size_t push(std::vector<MatrixView>& vs, size_t blksz) {
    const MatrixView uz = vs.back();
    auto zp = uz.zoomed_size_and_padding(0, blksz);
    vs.push_back(MatrixView{uz.offset, zp.second, zp.first});
    return uz.iter_size;
  }
  static void slide(std::vector<MatrixView>& vs, size_t i, size_t blksz) {
    const MatrixView uz = vs[vs.size() - 2];
    auto zp = uz.zoomed_size_and_padding(i, blksz);
    MatrixView& z = vs.back();
    z.iter_size = zp.first;
    z.padding = zp.second;
    z.offset = uz.offset + i;
  }
  static void split(std::vector<MatrixView>& vs, size_t start, size_t end, size_t cur) {
    const MatrixView uz = vs.back();
    const size_t pad = end <= cur ? 0 : end - cur;
    vs.push_back(MatrixView{uz.offset + start, pad, end - start});
  }

  T* buf_ = nullptr;
  size_t rs_ = 1, cs_ = 0;
  T alpha_ = T(1);
  std::vector<MatrixView> y_, x_;
  bool owner_ = false;
};

// ---------------------------------------------------------------------------
// ThreadInfo: a thread's id in its team and the team barrier
// (src/thread_comm.rs:112-136).
// ---------------------------------------------------------------------------
// Thrown by barrier() in every thread of a team that one of its threads has
// aborted, so that the whole team unwinds instead of waiting for a thread
// that left.
struct TeamAborted : std::runtime_error {
  TeamAborted() : std::runtime_error("thread team aborted") {}
};

class ThreadComm {
 public:
  explicit ThreadComm(size_t n) : n_(n) {}
  size_t size() const { return n_; }
  void barrier() {
    if (n_ == 1) return;
    std::unique_lock<std::mutex> lk(mu_);
    if (aborted_) throw TeamAborted();
    const uint64_t gen = gen_;
    if (++arrived_ == n_) {
      arrived_ = 0;
      ++gen_;
      cv_.notify_all();
    } else {
      cv_.wait(lk, [&] { return gen_ != gen || aborted_; });
      if (gen_ == gen) throw TeamAborted();
    }
  }
  // Wakes every waiter; this and every later barrier() throws TeamAborted.
  void abort() {
    std::lock_guard<std::mutex> lk(mu_);
    aborted_ = true;
    cv_.notify_all();
  }

 private:
  size_t n_;
  std::mutex mu_;
  std::condition_variable cv_;
  size_t arrived_ = 0;
  uint64_t gen_ = 0;
  bool aborted_ = false;
};

class ThreadInfo {
 public:
  ThreadInfo(size_t id, std::shared_ptr<ThreadComm> comm) : id_(id), comm_(std::move(comm)) {}
  static ThreadInfo single_thread() { return ThreadInfo(0, std::make_shared<ThreadComm>(1)); }
  size_t thread_id() const { return id_; }
  size_t num_threads() const { return comm_->size(); }
  void barrier() const { comm_->barrier(); }
  void abort_team() const { comm_->abort(); }

 private:
  size_t id_;
  std::shared_ptr<ThreadComm> comm_;
};

// ---------------------------------------------------------------------------
// Partitioners (src/composables/part.rs)
// ---------------------------------------------------------------------------
template <size_t Bsz, typename S>
struct PartM {
  S child;
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo& thr) {
    const size_t m_save = a.push_y_view(Bsz);
    c.push_y_view(Bsz);
    for (size_t i = 0; i < m_save; i += Bsz) {
      a.slide_y_view_to(i, Bsz);
      c.slide_y_view_to(i, Bsz);
      child.run(a, b, c, thr);
    }
    a.pop_y_view();
    c.pop_y_view();
  }
  static std::vector<AlgorithmStep> hierarchy_description() {
    auto d = S::hierarchy_description();
    d.push_back(AlgorithmStep{StepKind::M, Bsz});
    return d;
  }
};

template <size_t Bsz, typename S>
struct PartN {
  S child;
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo& thr) {
    const size_t n_save = b.push_x_view(Bsz);
    c.push_x_view(Bsz);
    for (size_t i = 0; i < n_save; i += Bsz) {
      b.slide_x_view_to(i, Bsz);
      c.slide_x_view_to(i, Bsz);
      child.run(a, b, c, thr);
    }
    b.pop_x_view();
    c.pop_x_view();
  }
  static std::vector<AlgorithmStep> hierarchy_description() {
    auto d = S::hierarchy_description();
    d.push_back(AlgorithmStep{StepKind::N, Bsz});
    return d;
  }
};

// The first k slab uses C's own scalar as beta, later slabs accumulate
// (beta = 1); the scalar is restored at the end (part.rs:96-110).
template <size_t Bsz, typename S>
struct PartK {
  S child;
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo& thr) {
    const size_t k_save = a.push_x_view(Bsz);
    b.push_y_view(Bsz);
    const auto beta_save = c.scalar();
    for (size_t i = 0; i < k_save; i += Bsz) {
      a.slide_x_view_to(i, Bsz);
      b.slide_y_view_to(i, Bsz);
      child.run(a, b, c, thr);
      c.set_scalar(1);
    }
    a.pop_x_view();
    b.pop_y_view();
    c.set_scalar(beta_save);
  }
  static std::vector<AlgorithmStep> hierarchy_description() {
    auto d = S::hierarchy_description();
    d.push_back(AlgorithmStep{StepKind::K, Bsz});
    return d;
  }
};

// ---------------------------------------------------------------------------
// SpawnThreads (src/composables/spawn.rs:100-135): runs the child on a team
// of threads, each with its own node and its own aliases of the operands,
// then a team barrier. A thread that throws aborts the team (the others
// leave at their next barrier) and the first error that is not TeamAborted
// is rethrown to the caller once every thread has joined.
// ---------------------------------------------------------------------------
template <typename S>
struct SpawnThreads {
  size_t n_threads = 1;
  std::vector<S> nodes = std::vector<S>(1);
  void set_n_threads(size_t n) {
    n_threads = std::max<size_t>(1, n);
    nodes.assign(n_threads, S());
  }
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo&) {
    auto comm = std::make_shared<ThreadComm>(n_threads);
    std::vector<std::thread> workers;
    std::vector<std::exception_ptr> errs(n_threads);
    std::vector<char> aborted(n_threads, 0);
    auto body = [&](size_t id, A& ma, B& mb, C& mc) {
      ThreadInfo thr(id, comm);
      try {
        nodes[id].run(ma, mb, mc, thr);
        thr.barrier();
      } catch (const TeamAborted&) {
        aborted[id] = 1;
      } catch (...) {
        errs[id] = std::current_exception();
        comm->abort();
      }
    };
    // the aliases are taken here, before thread 0 starts pushing views
    std::vector<A> as;
    std::vector<B> bs;
    std::vector<C> cs;
    for (size_t id = 1; id < n_threads; ++id) {
      as.push_back(a.alias());
      bs.push_back(b.alias());
      cs.push_back(c.alias());
    }
    for (size_t id = 1; id < n_threads; ++id)
      workers.emplace_back([&, id] { body(id, as[id - 1], bs[id - 1], cs[id - 1]); });
    body(0, a, b, c);
    for (auto& w : workers) w.join();
    for (auto& e : errs)
      if (e) std::rethrow_exception(e);
    for (char x : aborted)
      if (x) throw TeamAborted();
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return S::hierarchy_description(); }
};

// ---------------------------------------------------------------------------
// GpuGemm<T>: the GPU leaf. Thread 0 of the team computes
// C := beta*C + alpha*A*B on the current views with alpha = a.scalar*b.scalar
// and beta = c.scalar (src/kern/kernel_nm.rs:44-45) through momms_gemm; the
// rest of the team waits at the barrier.
// ---------------------------------------------------------------------------
template <typename T, int Precision = MOMMS_PREC_PLAIN>
struct GpuGemm {
  void* stream = nullptr;        // cudaStream_t; nullptr = legacy default stream
  double target_rel_err = 0.0;   // Ozaki only
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo& thr) {
    if (thr.thread_id() == 0) {
      momms_gemm_desc d;
      std::memset(&d, 0, sizeof(d));
      d.dtype = std::is_same<T, double>::value ? MOMMS_DTYPE_F64 : MOMMS_DTYPE_F32;
      d.precision = Precision;
      d.m = (int64_t)c.height();
      d.n = (int64_t)c.width();
      d.k = (int64_t)a.width();
      d.alpha = (double)(a.scalar() * b.scalar());
      d.beta = (double)c.scalar();
      d.a = momms_operand{(void*)a.buffer(), (int64_t)a.row_stride(), (int64_t)a.column_stride(), MOMMS_MEM_AUTO, 0};
      d.b = momms_operand{(void*)b.buffer(), (int64_t)b.row_stride(), (int64_t)b.column_stride(), MOMMS_MEM_AUTO, 0};
      d.c = momms_operand{(void*)c.buffer(), (int64_t)c.row_stride(), (int64_t)c.column_stride(), MOMMS_MEM_AUTO, 0};
      d.target_rel_err = target_rel_err;
      const int rc = momms_gemm(&d, stream);
      if (rc != MOMMS_OK) throw std::runtime_error(std::string("momms_gemm: ") + momms_last_error());
    }
    thr.barrier();
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return {}; }
};

}  // namespace momms
