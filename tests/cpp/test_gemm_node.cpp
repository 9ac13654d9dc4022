// Tests of include/momms/gemm_node.hpp.
//
//   test_gemm_node cpu          view arithmetic, partitioner call sequences,
//                               beta handling, thread teams (no GPU)
//   test_gemm_node gpu <dir>    composed algorithms with the GPU leaf; each case
//                               writes <dir>/<name>.bin for the Python side to
//                               check against the oracle
//
// Exit status 0 = all checks passed.
#include <momms/gemm_node.hpp>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>

using namespace momms;

static int g_failures = 0;
#define CHECK(...)                                                           \
  do {                                                                       \
    if (!(__VA_ARGS__)) {                                                        \
      std::fprintf(stderr, "%s:%d: CHECK failed: %s\n", __FILE__, __LINE__, #__VA_ARGS__); \
      ++g_failures;                                                          \
    }                                                                        \
  } while (0)

// ---------------------------------------------------------------------------
// CPU leaves used to test the composition layer
// ---------------------------------------------------------------------------

// C := beta*C + alpha*A*B on the current views, double accumulation.
struct NaiveLeaf {
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo&) {
    const double alpha = a.scalar() * b.scalar(), beta = c.scalar();
    for (size_t j = 0; j < c.width(); ++j)
      for (size_t i = 0; i < c.height(); ++i) {
        double s = 0;
        for (size_t p = 0; p < a.width(); ++p) s += (double)a.get(i, p) * (double)b.get(p, j);
        c.set(i, j, (typename std::decay<decltype(c.get(0, 0))>::type)(beta * c.get(i, j) + alpha * s));
      }
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return {}; }
};

// Records every call: offsets of the views into the base buffers, sizes, scalars.
struct Call {
  ptrdiff_t a_off, b_off, c_off;
  size_t m, n, k;
  double alpha, beta;
};
static std::vector<Call>* g_calls = nullptr;
static const double* g_base_a = nullptr;
static const double* g_base_b = nullptr;
static const double* g_base_c = nullptr;
struct RecordLeaf {
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo&) {
    g_calls->push_back(Call{a.buffer() - g_base_a, b.buffer() - g_base_b, c.buffer() - g_base_c, c.height(), c.width(),
                            a.width(), a.scalar() * b.scalar(), c.scalar()});
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return {}; }
};

// Each thread of the team takes a contiguous range of C's columns (the
// reference's ParallelN with an even split), then the team meets at a barrier.
struct TeamColumnsLeaf {
  template <typename A, typename B, typename C>
  void run(A& a, B& b, C& c, const ThreadInfo& thr) {
    const size_t n = c.width(), t = thr.num_threads(), id = thr.thread_id();
    const size_t lo = n * id / t, hi = n * (id + 1) / t;
    b.push_x_split(lo, hi);
    c.push_x_split(lo, hi);
    NaiveLeaf().run(a, b, c, thr);
    b.pop_x_split();
    c.pop_x_split();
    thr.barrier();
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return {}; }
};

// Thread 2 throws after `Rounds` team barriers; the others keep meeting at
// barriers and must be released by the team abort.
template <int Rounds>
struct ThrowOnThread2 {
  template <typename A, typename B, typename C>
  void run(A&, B&, C&, const ThreadInfo& thr) {
    for (int r = 0; r < 10; ++r) {
      if (r == Rounds && thr.thread_id() == 2) throw std::runtime_error("planted");
      thr.barrier();
    }
  }
  static std::vector<AlgorithmStep> hierarchy_description() { return {}; }
};

template <typename T>
static double max_abs_diff(const Matrix<T>& x, const Matrix<T>& y) {
  double d = 0;
  for (size_t j = 0; j < x.width(); ++j)
    for (size_t i = 0; i < x.height(); ++i) d = std::max(d, std::fabs((double)x.get(i, j) - (double)y.get(i, j)));
  return d;
}

template <typename T>
static void copy_into(Matrix<T>& dst, const Matrix<T>& src) {
  for (size_t j = 0; j < src.width(); ++j)
    for (size_t i = 0; i < src.height(); ++i) dst.set(i, j, src.get(i, j));
}

// ---------------------------------------------------------------------------
// CPU checks
// ---------------------------------------------------------------------------
static void test_views() {
  // zoomed_size_and_padding: block of 4 over an unpadded 10 -> 4,4,2
  MatrixView v{0, 0, 10};
  CHECK(v.zoomed_size_and_padding(0, 4) == std::make_pair<size_t, size_t>(4, 0));
  CHECK(v.zoomed_size_and_padding(8, 4) == std::make_pair<size_t, size_t>(2, 0));
  // a view of iter 12 with 3 padding (physical 9): the block at 8 has iter
  // size 4 of which 3 are padding, the block at 4 is fully physical
  MatrixView p{0, 3, 12};
  CHECK(p.physical_size() == 9);
  CHECK(p.zoomed_size_and_padding(8, 4) == std::make_pair<size_t, size_t>(4, 3));
  CHECK(p.zoomed_size_and_padding(4, 4) == std::make_pair<size_t, size_t>(4, 0));
  // a block entirely inside the padding
  MatrixView q{0, 6, 8};
  CHECK(q.zoomed_size_and_padding(4, 4) == std::make_pair<size_t, size_t>(4, 4));
  MatrixView e{0, 9, 8};
  CHECK(e.physical_size() == 0);

  Matrix<double> m(10, 7);
  for (size_t j = 0; j < 7; ++j)
    for (size_t i = 0; i < 10; ++i) m.set(i, j, 100.0 * i + j);
  CHECK(m.row_stride() == 1 && m.column_stride() == 10);
  CHECK(m.push_y_view(4) == 10);
  CHECK(m.height() == 4 && m.width() == 7);
  m.slide_y_view_to(8, 4);
  CHECK(m.height() == 2 && m.get(0, 0) == 800.0 && m.get(1, 6) == 906.0);
  CHECK(m.push_x_view(3) == 7);
  m.slide_x_view_to(6, 3);
  CHECK(m.width() == 1 && m.get(1, 0) == 906.0);
  m.pop_x_view();
  m.pop_y_view();
  CHECK(m.height() == 10 && m.width() == 7 && m.get(9, 6) == 906.0);

  // split past the end pads the view (general_stride.rs:104-114)
  m.push_y_split(6, 12);
  CHECK(m.iter_height() == 6 && m.height() == 4 && m.get(0, 0) == 600.0);
  m.pop_y_split();

  m.transpose();
  CHECK(m.height() == 7 && m.width() == 10 && m.get(6, 9) == 906.0 && m.row_stride() == 10);
  bool threw = false;
  m.push_y_view(2);
  try {
    m.transpose();
  } catch (const std::logic_error&) {
    threw = true;
  }
  CHECK(threw);
  m.pop_y_view();

  auto al = m.alias();
  CHECK(al.height() == 7 && al.get(6, 9) == 906.0 && al.buffer() == m.buffer());
}

static void test_hierarchy() {
  using Algo = SpawnThreads<PartN<3000, PartK<192, PartM<120, GpuGemm<double>>>>>;
  auto d = Algo::hierarchy_description();
  // innermost first (part.rs: the child's description, then this step)
  CHECK(d.size() == 3);
  CHECK(d[0] == (AlgorithmStep{StepKind::M, 120}));
  CHECK(d[1] == (AlgorithmStep{StepKind::K, 192}));
  CHECK(d[2] == (AlgorithmStep{StepKind::N, 3000}));
}

static void test_call_sequence() {
  // PartN<4, PartK<5, PartM<3, Record>>> on m=7, n=6, k=11
  Matrix<double> a(7, 11), b(11, 6), c(7, 6);
  std::vector<Call> calls;
  g_calls = &calls;
  g_base_a = a.buffer();
  g_base_b = b.buffer();
  g_base_c = c.buffer();
  a.set_scalar(2.0);
  b.set_scalar(-0.5);
  c.set_scalar(0.25);
  PartN<4, PartK<5, PartM<3, RecordLeaf>>> algo;
  algo.run(a, b, c, ThreadInfo::single_thread());
  // 2 column blocks x 3 k slabs x 3 row blocks
  CHECK(calls.size() == 18);
  size_t idx = 0;
  for (size_t jn = 0; jn < 6; jn += 4)
    for (size_t pk = 0; pk < 11; pk += 5)
      for (size_t im = 0; im < 7; im += 3) {
        const Call& cl = calls[idx++];
        CHECK(cl.m == std::min<size_t>(3, 7 - im));
        CHECK(cl.n == std::min<size_t>(4, 6 - jn));
        CHECK(cl.k == std::min<size_t>(5, 11 - pk));
        CHECK(cl.a_off == (ptrdiff_t)(im + pk * 7));
        CHECK(cl.b_off == (ptrdiff_t)(pk + jn * 11));
        CHECK(cl.c_off == (ptrdiff_t)(im + jn * 7));
        CHECK(cl.alpha == -1.0);
        // the first k slab of each column block uses C's scalar, later ones 1
        CHECK(cl.beta == (pk == 0 ? 0.25 : 1.0));
      }
  CHECK(c.scalar() == 0.25);
  CHECK(a.height() == 7 && a.width() == 11 && b.width() == 6 && c.width() == 6);
  g_calls = nullptr;
}

static void test_composed_numerics() {
  const size_t m = 37, n = 29, k = 53;
  Matrix<double> a(m, k), b(n, k), c(m, n), c_ref(m, n);
  a.fill_rand(1);
  b.fill_rand(2);
  b.transpose();  // B stored row-major (k x n view of an n x k matrix)
  c.fill_rand(3);
  copy_into(c_ref, c);
  a.set_scalar(1.5);
  c.set_scalar(-0.75);
  c_ref.set_scalar(-0.75);
  NaiveLeaf().run(a, b, c_ref, ThreadInfo::single_thread());
  PartM<8, PartK<10, PartN<7, NaiveLeaf>>> algo;
  algo.run(a, b, c, ThreadInfo::single_thread());
  CHECK(max_abs_diff(c, c_ref) < 1e-12);
  CHECK(c.scalar() == -0.75);
}

static void test_teams() {
  const size_t m = 40, n = 33, k = 17;
  Matrix<double> a(m, k), b(k, n), c(m, n), c_ref(m, n);
  a.fill_rand(4);
  b.fill_rand(5);
  c.fill_rand(6);
  copy_into(c_ref, c);
  NaiveLeaf().run(a, b, c_ref, ThreadInfo::single_thread());
  SpawnThreads<PartK<6, TeamColumnsLeaf>> algo;
  algo.set_n_threads(4);
  algo.run(a, b, c, ThreadInfo::single_thread());
  CHECK(max_abs_diff(c, c_ref) < 1e-12);

  // many barrier rounds on a larger team
  auto comm = std::make_shared<ThreadComm>(6);
  std::atomic<int> counter{0};
  std::vector<std::thread> ts;
  bool ok = true;
  std::mutex mu;
  for (size_t id = 0; id < 6; ++id)
    ts.emplace_back([&, id] {
      ThreadInfo thr(id, comm);
      for (int r = 0; r < 200; ++r) {
        counter.fetch_add(1);
        thr.barrier();
        if (counter.load() != 6 * (r + 1)) {
          std::lock_guard<std::mutex> g(mu);
          ok = false;
        }
        thr.barrier();
      }
    });
  for (auto& t : ts) t.join();
  CHECK(ok);

  // an exception on one worker reaches the caller, after the team is joined
  auto planted = [&](auto algo) {
    algo.set_n_threads(4);
    try {
      algo.run(a, b, c, ThreadInfo::single_thread());
    } catch (const TeamAborted&) {
      return false;
    } catch (const std::runtime_error& e) {
      return std::string(e.what()) == "planted";
    }
    return false;
  };
  CHECK(planted(SpawnThreads<ThrowOnThread2<0>>()));
  CHECK(planted(SpawnThreads<ThrowOnThread2<3>>()));
}

// ---------------------------------------------------------------------------
// GPU cases: run a composed algorithm, dump operands and result
// ---------------------------------------------------------------------------
template <typename T>
static void dump(const std::string& path, int precision, const Matrix<T>& a, const Matrix<T>& b, const Matrix<T>& c0,
                 const Matrix<T>& c) {
  std::ofstream f(path, std::ios::binary);
  const int64_t hdr[5] = {std::is_same<T, double>::value ? 0 : 1, precision, (int64_t)c.height(), (int64_t)c.width(),
                          (int64_t)a.width()};
  const double sc[2] = {(double)(a.scalar() * b.scalar()), (double)c.scalar()};
  f.write((const char*)hdr, sizeof(hdr));
  f.write((const char*)sc, sizeof(sc));
  auto put = [&](const Matrix<T>& x) {
    for (size_t j = 0; j < x.width(); ++j)
      for (size_t i = 0; i < x.height(); ++i) {
        const T v = x.get(i, j);
        f.write((const char*)&v, sizeof(T));
      }
  };
  put(a);
  put(b);
  put(c0);
  put(c);
}

template <typename T, typename Algo>
static void gpu_case(const std::string& dir, const std::string& name, int precision, size_t m, size_t n, size_t k,
                     bool transpose_b, T a_scalar, T b_scalar, T c_scalar, Algo& algo, uint64_t seed) {
  Matrix<T> a(m, k), b(transpose_b ? n : k, transpose_b ? k : n), c(m, n), c0(m, n);
  a.fill_rand(seed);
  b.fill_rand(seed + 1);
  if (transpose_b) b.transpose();
  c.fill_rand(seed + 2);
  copy_into(c0, c);
  a.set_scalar(a_scalar);
  b.set_scalar(b_scalar);
  c.set_scalar(c_scalar);
  c0.set_scalar(c_scalar);
  algo.run(a, b, c, ThreadInfo::single_thread());
  CHECK(c.scalar() == c_scalar);
  dump(dir + "/" + name + ".bin", precision, a, b, c0, c);
}

static int run_gpu(const std::string& dir) {
  {
    PartN<300, PartK<256, PartM<200, GpuGemm<double>>>> algo;
    gpu_case<double>(dir, "f64_nkm", MOMMS_PREC_PLAIN, 517, 611, 700, true, 0.5, -2.0, 0.25, algo, 11);
  }
  {
    // the reference's out-of-core blocking shape, on a team of 4 threads
    SpawnThreads<PartM<400, PartN<350, GpuGemm<double>>>> algo;
    algo.set_n_threads(4);
    gpu_case<double>(dir, "f64_spawn_mn", MOMMS_PREC_PLAIN, 1000, 900, 800, false, 1.0, 1.0, 1.0, algo, 21);
  }
  {
    PartK<512, GpuGemm<double, MOMMS_PREC_OZAKI>> algo;
    gpu_case<double>(dir, "f64_ozaki_k", MOMMS_PREC_OZAKI, 640, 480, 1300, false, 1.0, 1.0, 0.5, algo, 31);
  }
  {
    PartM<128, PartN<100, GpuGemm<float>>> algo;
    gpu_case<float>(dir, "f32_mn", MOMMS_PREC_PLAIN, 333, 250, 190, true, 1.0f, 0.75f, -1.0f, algo, 41);
  }
  {
    PartK<64, GpuGemm<float, MOMMS_PREC_SPLIT_TF32>> algo;
    gpu_case<float>(dir, "f32_tf32_k", MOMMS_PREC_SPLIT_TF32, 256, 384, 200, false, 1.0f, 1.0f, 1.0f, algo, 51);
  }
  // a failing leaf call surfaces as an exception, not a silent skip: f32 with
  // the f64-only Ozaki precision is rejected by the library
  {
    PartM<64, GpuGemm<float, MOMMS_PREC_OZAKI>> algo;
    Matrix<float> a(70, 10), b(10, 5), c(70, 5);
    a.fill_zero();
    b.fill_zero();
    c.fill_zero();
    bool threw = false;
    try {
      algo.run(a, b, c, ThreadInfo::single_thread());
    } catch (const std::runtime_error&) {
      threw = true;
    }
    CHECK(threw);
  }
  return 0;
}

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "cpu";
  try {
    if (mode == "cpu") {
      test_views();
      test_hierarchy();
      test_call_sequence();
      test_composed_numerics();
      test_teams();
    } else if (mode == "gpu" && argc > 2) {
      run_gpu(argv[2]);
    } else {
      std::fprintf(stderr, "usage: %s cpu | gpu <dir>\n", argv[0]);
      return 2;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "uncaught: %s\n", e.what());
    return 1;
  }
  if (g_failures) {
    std::fprintf(stderr, "%d check(s) failed\n", g_failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
