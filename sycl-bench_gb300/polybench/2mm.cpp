// Polybench_2mm: C += A*B, then E = C*D over N x N matrices (--size).
// Drop-in for sycl-bench polybench/2mm.cpp: same name, initialisation, host
// verification loop and CSV columns; each stage is a libgbpoly contraction
// (stage 1 accumulates into the pre-initialised C, beta = 1; stage 2 writes E).
#include <string>
#include <vector>

#include "polybench_common.h"

// 2mm.cpp:16-45
template <class T>
void init_array(T* A, T* B, T* C, T* D, size_t size) {
  const auto NI = size, NJ = size, NK = size, NL = size;
  for(size_t i = 0; i < NI; i++)
    for(size_t j = 0; j < NK; j++) A[i * NI + j] = ((T)i * j) / NI;
  for(size_t i = 0; i < NK; i++)
    for(size_t j = 0; j < NJ; j++) B[i * NK + j] = ((T)i * (j + 1)) / NJ;
  for(size_t i = 0; i < NL; i++)
    for(size_t j = 0; j < NJ; j++) C[i * NL + j] = ((T)i * (j + 3)) / NL;
  for(size_t i = 0; i < NI; i++)
    for(size_t j = 0; j < NL; j++) D[i * NL + j] = ((T)i * (j + 2)) / NK;
}

// Host oracle, 2mm.cpp:47-69 (C is updated in place, as in the reference).
template <class T>
void mm2_cpu(const T* A, const T* B, T* C, const T* D, T* E, size_t size) {
  const long NI = long(size);
  const size_t NJ = size, NK = size, NL = size;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++)
    for(size_t j = 0; j < NJ; j++)
      for(size_t k = 0; k < NK; ++k) C[i * NJ + j] += A[i * NK + k] * B[k * NJ + j];
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++)
    for(size_t j = 0; j < NL; j++) {
      E[i * NL + j] = 0;
      for(size_t k = 0; k < NJ; ++k) E[i * NL + j] += C[i * NJ + k] * D[k * NL + j];
    }
}

template <class T>
class Polybench_2mm {
public:
  Polybench_2mm(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), opt(poly::options(args, prec)),
        use_graph(args.cli.isFlagSet("--graph") && !args.device_queue.is_host()) {}

  ~Polybench_2mm() {
    if(graph) gbpoly_graph_destroy(args.device_queue.ctx(), graph);
  }

  void setup() {
    const size_t nn = size * size;
    A.resize(nn);
    B.resize(nn);
    C.resize(nn);
    D.resize(nn);
    E.resize(nn);
    make_inputs(A.data(), B.data(), C.data(), D.data());
    A_buffer.initialize(args.device_queue, A.data(), nn);
    B_buffer.initialize(args.device_queue, B.data(), nn);
    C_buffer.initialize(args.device_queue, C.data(), nn);
    D_buffer.initialize(args.device_queue, D.data(), nn);
    E_buffer.initialize(args.device_queue, E.data(), nn);
    if(use_graph) capture_stages();
  }

  void run(std::vector<gb::Event>& events) {
    if(use_graph) {  // both stages as one graph launch
      events.push_back(args.device_queue.submit(
          [&](gb::Handler& h) { gb::check(gbpoly_graph_launch(h.ctx(), graph), "graph launch"); }));
      return;
    }
    // C += A.B   (2mm.cpp:99-106)
    events.push_back(args.device_queue.submit([&](gb::Handler& h) { stage1(h); }));
    // E = C.D    (2mm.cpp:114-122)
    events.push_back(args.device_queue.submit([&](gb::Handler& h) { stage2(h); }));
  }

  bool verify(VerificationSetting&) {
    const size_t nn = size * size;
    const T* E_dev = E_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto E_cpu = poly::memo<T>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<T> a(nn), b(nn), c(nn), d(nn), e(nn);
        make_inputs(a.data(), b.data(), c.data(), d.data());
        mm2_cpu(a.data(), b.data(), c.data(), d.data(), e.data(), size);
        return e;
      });
      ok = poly::compare(E_cpu->data(), E_dev, nn);
    }
    if(opt.fp64_oracle || !opt.error_report.empty()) {
      auto ref = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] { return fp64_reference(); });
      if(opt.fp64_oracle) ok = poly::compare(ref->data(), E_dev, nn);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(E_dev, ref->data(), nn), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<T>("Polybench_2mm", opt) + (use_graph ? "_graph" : "");
  }

  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {4.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void stage1(gb::Handler& h) { contract(h, A_buffer.get(), B_buffer.get(), T(1), C_buffer.get()); }
  void stage2(gb::Handler& h) { contract(h, C_buffer.get(), D_buffer.get(), T(0), E_buffer.get()); }

  // --graph: record both stages into one CUDA graph (untimed, in setup)
  void capture_stages() {
    gbpoly_ctx* ctx = args.device_queue.ctx();
    if constexpr(std::is_same<T, float>::value) {
      size_t ws = 0;
      const int64_t n = int64_t(size);
      gb::check(gbpoly_workspace_query(opt.precision, n, n, n, 0, &ws), "workspace query");
      gb::check(gbpoly_workspace_reserve(ctx, ws), "workspace reserve");
    }
    gb::Handler h(args.device_queue);
    gb::check(gbpoly_graph_begin(ctx), "graph begin");
    stage1(h);
    stage2(h);
    gb::check(gbpoly_graph_end(ctx, &graph), "graph end");
  }

  // out = a.b + beta*out on the queue's device
  void contract(gb::Handler& h, const T* a, const T* b, T beta, T* out) {
    if(h.on_host()) {
      poly::host_gemm_body<T>(size, false, T(1), a, b, beta, out);
      return;
    }
    const int64_t n = int64_t(size);
    if constexpr(std::is_same<T, float>::value)
      gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.f, a, n, b, n, beta, out, n),
          "gemm");
    else
      gb::check(gbpoly_gemm_f64(h.ctx(), GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.0, a, n, b, n, beta, out, n), "gemm");
  }

  void make_inputs(T* a, T* b, T* c, T* d) const {
    if(opt.init == poly::Init::Polybench) {
      init_array(a, b, c, d, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(b, size * size, opt.init, opt.seed, 1);
      poly::fill_random(c, size * size, opt.init, opt.seed, 2);
      poly::fill_random(d, size * size, opt.init, opt.seed, 3);
    }
  }

  std::vector<double> fp64_reference() const {
    const size_t nn = size * size;
    std::vector<T> a(nn), b(nn), c(nn), d(nn);
    make_inputs(a.data(), b.data(), c.data(), d.data());
    if(args.device_queue.is_host()) {
      std::vector<double> c64(c.begin(), c.end()), e(nn, 0.0);
      poly::host_gemm_f64(size, false, false, 1.0, a.data(), b.data(), 1.0, c64);
      std::vector<double> d64(d.begin(), d.end());
      poly::host_gemm_f64(size, false, false, 1.0, c64.data(), d64.data(), 0.0, e);
      return e;
    }
    poly::Fp64Device dev(args.device_queue, size);
    double *dA = dev.upload(a.data()), *dB = dev.upload(b.data()), *dC = dev.upload(c.data());
    double *dD = dev.upload(d.data()), *dE = dev.zeros();
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dA, dB, 1.0, dC);
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dC, dD, 0.0, dE);
    return dev.download(dE);
  }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  bool use_graph;
  gbpoly_graph* graph = nullptr;
  std::vector<T> A, B, C, D, E;
  PrefetchedBuffer<T, 2> A_buffer, B_buffer, C_buffer, D_buffer, E_buffer;
};

int main(int argc, char** argv) {
  BenchmarkApp app(argc, argv);
  if(!app.getArgs().device_queue.valid()) return 0;
  std::vector<gbpoly_precision> forms;
  try {
    forms = poly::precisions(app.getArgs());
  } catch(std::exception& e) {
    std::cerr << "Error: " << e.what() << std::endl;
    return 0;
  }
  for(auto p : forms) app.run<Polybench_2mm<float>>(p);
  if constexpr(SYCL_BENCH_HAS_FP64_SUPPORT) app.run<Polybench_2mm<double>>();
  return 0;
}
