// Polybench_3mm: E = A*B, F = C*D, G = E*F over N x N matrices (--size).
// Drop-in for sycl-bench polybench/3mm.cpp: same name, initialisation, host
// verification loop and CSV columns; each stage is a libgbpoly contraction.
// The reference accumulates each stage onto zero-initialised E, F, G; the
// stages here write their output (beta = 0), which is the same value.
// Options beyond the reference's: --graph (the stages as one captured CUDA
// graph) and --grouped (E and F, which are independent, as one grouped
// launch; the float benchmark only).
#include <string>
#include <vector>

#include "polybench_common.h"

// 3mm.cpp:17-47
template <class T>
void init_array(T* A, T* B, T* C, T* D, size_t size) {
  const auto NI = size, NJ = size, NK = size, NL = size, NM = size;
  for(size_t i = 0; i < NI; i++)
    for(size_t j = 0; j < NK; j++) A[i * NK + j] = ((T)i * j) / NI;
  for(size_t i = 0; i < NK; i++)
    for(size_t j = 0; j < NJ; j++) B[i * NJ + j] = ((T)i * (j + 1)) / NJ;
  for(size_t i = 0; i < NJ; i++)
    for(size_t j = 0; j < NM; j++) C[i * NM + j] = ((T)i * (j + 3)) / NL;
  for(size_t i = 0; i < NM; i++)
    for(size_t j = 0; j < NL; j++) D[i * NL + j] = ((T)i * (j + 2)) / NK;
}

// Host oracle, 3mm.cpp:49-86.
template <class T>
void mm3_cpu(const T* A, const T* B, const T* C, const T* D, T* E, T* F, T* G, size_t size) {
  const long NI = long(size);
  const size_t NJ = size, NK = size, NL = size, NM = size;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++)
    for(size_t j = 0; j < NJ; j++) {
      E[i * NJ + j] = 0;
      for(size_t k = 0; k < NK; ++k) E[i * NJ + j] += A[i * NK + k] * B[k * NJ + j];
    }
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++)
    for(size_t j = 0; j < NL; j++) {
      F[i * NL + j] = 0;
      for(size_t k = 0; k < NM; ++k) F[i * NL + j] += C[i * NM + k] * D[k * NL + j];
    }
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++)
    for(size_t j = 0; j < NL; j++) {
      G[i * NL + j] = 0;
      for(size_t k = 0; k < NJ; ++k) G[i * NL + j] += E[i * NJ + k] * F[k * NL + j];
    }
}

template <class T>
class Polybench_3mm {
public:
  Polybench_3mm(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), opt(poly::options(args, prec)),
        use_graph(args.cli.isFlagSet("--graph") && !args.device_queue.is_host()),
        use_grouped(std::is_same<T, float>::value && args.cli.isFlagSet("--grouped") &&
                    !args.device_queue.is_host()) {}

  ~Polybench_3mm() {
    if(graph) gbpoly_graph_destroy(args.device_queue.ctx(), graph);
    if(grouped) gbpoly_grouped_destroy(args.device_queue.ctx(), grouped);
  }

  void setup() {
    const size_t nn = size * size;
    for(auto* v : {&A, &B, &C, &D, &E, &F, &G}) v->resize(nn);
    make_inputs(A.data(), B.data(), C.data(), D.data());
    A_buffer.initialize(args.device_queue, A.data(), nn);
    B_buffer.initialize(args.device_queue, B.data(), nn);
    C_buffer.initialize(args.device_queue, C.data(), nn);
    D_buffer.initialize(args.device_queue, D.data(), nn);
    E_buffer.initialize(args.device_queue, E.data(), nn);
    F_buffer.initialize(args.device_queue, F.data(), nn);
    G_buffer.initialize(args.device_queue, G.data(), nn);
    if(use_grouped) plan_grouped();
    if(use_graph) capture_stages();
  }

  void run(std::vector<gb::Event>& events) {
    if(use_graph) {  // the three stages as one graph launch
      events.push_back(args.device_queue.submit(
          [&](gb::Handler& h) { gb::check(gbpoly_graph_launch(h.ctx(), graph), "graph launch"); }));
      return;
    }
    if(use_grouped) {  // E and F, which are independent, as one grouped launch
      events.push_back(args.device_queue.submit(
          [&](gb::Handler& h) { gb::check(gbpoly_grouped_run(h.ctx(), grouped), "grouped run"); }));
    } else {
      events.push_back(args.device_queue.submit([&](gb::Handler& h) { stage(h, 0); }));  // E = A.B (3mm.cpp:120-127)
      events.push_back(args.device_queue.submit([&](gb::Handler& h) { stage(h, 1); }));  // F = C.D (3mm.cpp:135-142)
    }
    events.push_back(args.device_queue.submit([&](gb::Handler& h) { stage(h, 2); }));  // G = E.F (3mm.cpp:150-157)
  }

  bool verify(VerificationSetting&) {
    const size_t nn = size * size;
    const T* G_dev = G_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto G_cpu = poly::memo<T>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<T> a(nn), b(nn), c(nn), d(nn), e(nn), f(nn), g(nn);
        make_inputs(a.data(), b.data(), c.data(), d.data());
        mm3_cpu(a.data(), b.data(), c.data(), d.data(), e.data(), f.data(), g.data(), size);
        return g;
      });
      ok = poly::compare(G_cpu->data(), G_dev, nn);
    }
    if(opt.fp64_oracle || !opt.error_report.empty()) {
      auto ref = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] { return fp64_reference(); });
      if(opt.fp64_oracle) ok = poly::compare(ref->data(), G_dev, nn);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(G_dev, ref->data(), nn), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<T>("Polybench_3mm", opt) + (use_grouped ? "_grouped" : "") + (use_graph ? "_graph" : "");
  }

  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {6.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void stage(gb::Handler& h, int i) {
    if(i == 0) contract(h, A_buffer.get(), B_buffer.get(), E_buffer.get());
    if(i == 1) contract(h, C_buffer.get(), D_buffer.get(), F_buffer.get());
    if(i == 2) contract(h, E_buffer.get(), F_buffer.get(), G_buffer.get());
  }

  // --graph: record the three stages into one CUDA graph (untimed, in setup)
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
    if(use_grouped)
      gb::check(gbpoly_grouped_run(ctx, grouped), "grouped run");
    else
      for(int i = 0; i < 2; ++i) stage(h, i);
    stage(h, 2);
    gb::check(gbpoly_graph_end(ctx, &graph), "graph end");
  }

  // --grouped: E = A.B and F = C.D as one plan (untimed, in setup)
  void plan_grouped() {
    if constexpr(std::is_same<T, float>::value) {
      const int64_t n = int64_t(size);
      gbpoly_gemm_desc d[2] = {};
      const T* ops[2][2] = {{A_buffer.get(), B_buffer.get()}, {C_buffer.get(), D_buffer.get()}};
      T* outs[2] = {E_buffer.get(), F_buffer.get()};
      for(int i = 0; i < 2; ++i) {
        d[i].op_a = d[i].op_b = GBPOLY_OP_N;
        d[i].M = d[i].N = d[i].K = n;
        d[i].alpha = 1.f;
        d[i].beta = 0.f;
        d[i].A = ops[i][0], d[i].lda = n;
        d[i].B = ops[i][1], d[i].ldb = n;
        d[i].C = outs[i], d[i].ldc = n;
      }
      gb::check(gbpoly_grouped_plan(args.device_queue.ctx(), opt.precision, d, 2, &grouped), "grouped plan");
    }
  }

  void contract(gb::Handler& h, const T* a, const T* b, T* out) {
    if(h.on_host()) {
      poly::host_gemm_body<T>(size, false, T(1), a, b, T(0), out);
      return;
    }
    const int64_t n = int64_t(size);
    if constexpr(std::is_same<T, float>::value)
      gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.f, a, n, b, n, 0.f, out, n),
          "gemm");
    else
      gb::check(gbpoly_gemm_f64(h.ctx(), GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.0, a, n, b, n, 0.0, out, n), "gemm");
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
      std::vector<double> e(nn, 0.0), f(nn, 0.0), g(nn, 0.0);
      poly::host_gemm_f64(size, false, false, 1.0, a.data(), b.data(), 0.0, e);
      poly::host_gemm_f64(size, false, false, 1.0, c.data(), d.data(), 0.0, f);
      poly::host_gemm_f64(size, false, false, 1.0, e.data(), f.data(), 0.0, g);
      return g;
    }
    poly::Fp64Device dev(args.device_queue, size);
    double *dA = dev.upload(a.data()), *dB = dev.upload(b.data()), *dC = dev.upload(c.data());
    double *dD = dev.upload(d.data()), *dE = dev.zeros(), *dF = dev.zeros(), *dG = dev.zeros();
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dA, dB, 0.0, dE);
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dC, dD, 0.0, dF);
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dE, dF, 0.0, dG);
    return dev.download(dG);
  }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  bool use_graph, use_grouped;
  gbpoly_graph* graph = nullptr;
  gbpoly_grouped* grouped = nullptr;
  std::vector<T> A, B, C, D, E, F, G;
  PrefetchedBuffer<T, 2> A_buffer, B_buffer, C_buffer, D_buffer, E_buffer, F_buffer, G_buffer;
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
  for(auto p : forms) app.run<Polybench_3mm<float>>(p);
  if constexpr(SYCL_BENCH_HAS_FP64_SUPPORT) app.run<Polybench_3mm<double>>();
  return 0;
}
