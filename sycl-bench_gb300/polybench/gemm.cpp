// Polybench_Gemm: C = beta*C + alpha*A*B over N x N matrices (NI=NJ=NK=--size),
// alpha=32412, beta=2123.  Drop-in for sycl-bench polybench/gemm.cpp: same
// name, initialisation, host verification loop and CSV columns; the device
// kernel is libgbpoly's contraction, --precision selects its form.
#include <string>
#include <vector>

#include "polybench_common.h"

#define ALPHA 32412
#define BETA 2123

// gemm.cpp:18-40.  (T)i * j promotes j to T; the division by size likewise.
template <class T>
void init(T* A, T* B, T* C, size_t size) {
  const auto NI = size, NJ = size, NK = size;
  for(size_t i = 0; i < NI; i++)
    for(size_t j = 0; j < NK; j++) A[i * NK + j] = ((T)i * j) / NI;
  for(size_t i = 0; i < NK; i++)
    for(size_t j = 0; j < NJ; j++) B[i * NJ + j] = ((T)i * j + 1) / NJ;
  for(size_t i = 0; i < NI; i++)
    for(size_t j = 0; j < NJ; j++) C[i * NJ + j] = ((T)i * j + 2) / NJ;
}

// Host oracle, gemm.cpp:42-56: per element, scale by beta then accumulate
// alpha*A*B in k order.  Rows run in parallel; each element's operation order
// is the reference's, so the result does not depend on the thread count.
template <class T>
void gemm(const T* A, const T* B, T* C, size_t size, T alpha, T beta) {
  const long NI = long(size);
  const size_t NJ = size, NK = size;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < NI; i++) {
    for(size_t j = 0; j < NJ; j++) {
      C[i * NJ + j] *= beta;
      for(size_t k = 0; k < NK; ++k) C[i * NJ + j] += alpha * A[i * NK + k] * B[k * NJ + j];
    }
  }
}

template <class T>
class Polybench_Gemm {
public:
  Polybench_Gemm(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), opt(poly::options(args, prec)) {
    alpha = opt.has_alpha ? T(opt.alpha) : T(ALPHA);
    beta = opt.has_beta ? T(opt.beta) : T(BETA);
  }

  void setup() {
    A.resize(size * size);
    B.resize(size * size);
    C.resize(size * size);
    make_inputs(A.data(), B.data(), C.data());
    A_buffer.initialize(args.device_queue, A.data(), size * size);
    B_buffer.initialize(args.device_queue, B.data(), size * size);
    C_buffer.initialize(args.device_queue, C.data(), size * size);
  }

  void run(std::vector<gb::Event>& events) {
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) {
        poly::host_gemm_body<T>(size, false, alpha, A_buffer.get(), B_buffer.get(), beta, C_buffer.get());
        return;
      }
      const int64_t n = int64_t(size);
      if constexpr(std::is_same<T, float>::value)
        gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, alpha, A_buffer.get(), n,
                      B_buffer.get(), n, beta, C_buffer.get(), n),
            "gemm");
      else
        gb::check(gbpoly_gemm_f64(h.ctx(), GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, alpha, A_buffer.get(), n,
                      B_buffer.get(), n, beta, C_buffer.get(), n),
            "gemm");
    }));
  }

  bool verify(VerificationSetting&) {
    const size_t nn = size * size;
    const T* C_dev = C_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto C_cpu = poly::memo<T>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<T> a(nn), b(nn), c(nn);
        make_inputs(a.data(), b.data(), c.data());
        gemm(a.data(), b.data(), c.data(), size, alpha, beta);
        return c;
      });
      ok = poly::compare(C_cpu->data(), C_dev, nn);
    }
    if(opt.fp64_oracle || !opt.error_report.empty()) {
      auto ref = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] { return fp64_reference(); });
      if(opt.fp64_oracle) ok = poly::compare(ref->data(), C_dev, nn);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(C_dev, ref->data(), nn), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<T>("Polybench_Gemm", opt);
  }

  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {2.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void make_inputs(T* a, T* b, T* c) const {
    if(opt.init == poly::Init::Polybench) {
      init(a, b, c, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(b, size * size, opt.init, opt.seed, 1);
      poly::fill_random(c, size * size, opt.init, opt.seed, 2);
    }
  }

  std::vector<double> fp64_reference() const {
    const size_t nn = size * size;
    std::vector<T> a(nn), b(nn), c(nn);
    make_inputs(a.data(), b.data(), c.data());
    if(args.device_queue.is_host()) {
      std::vector<double> r(c.begin(), c.end());
      poly::host_gemm_f64(size, false, false, double(alpha), a.data(), b.data(), double(beta), r);
      return r;
    }
    poly::Fp64Device d(args.device_queue, size);
    double *dA = d.upload(a.data()), *dB = d.upload(b.data()), *dC = d.upload(c.data());
    d.gemm(GBPOLY_OP_N, GBPOLY_OP_N, double(alpha), dA, dB, double(beta), dC);
    return d.download(dC);
  }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  T alpha, beta;
  std::vector<T> A, B, C;
  PrefetchedBuffer<T, 2> A_buffer, B_buffer, C_buffer;
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
  for(auto p : forms) app.run<Polybench_Gemm<float>>(p);
  if constexpr(SYCL_BENCH_HAS_FP64_SUPPORT) app.run<Polybench_Gemm<double>>();
  return 0;
}
