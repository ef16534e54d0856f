// Polybench_Syrk: C = beta*C + alpha*A*A^T over the full N x N square
// (N = M = --size), alpha=123, beta=14512.  Drop-in for sycl-bench
// polybench/syrk.cpp: same name, initialisation, host verification loop and
// CSV columns; the device kernel is libgbpoly's symmetric rank-k update.
#include <string>
#include <vector>

#include "polybench_common.h"

// syrk.cpp:18-31
template <class T>
void init_arrays(T* A, T* C, size_t size) {
  const auto N = size, M = size;
  for(size_t i = 0; i < N; i++) {
    for(size_t j = 0; j < M; j++) A[i * M + j] = ((T)i * j) / N;
    for(size_t j = 0; j < N; j++) C[i * M + j] = ((T)i * j + 2) / N;
  }
}

// Host oracle, syrk.cpp:33-51 (rows in parallel, each element in k order).
template <class T>
void syrk(const T* A, T* C, size_t size, T alpha, T beta) {
  const long N = long(size);
  const size_t M = size;
  for(long i = 0; i < N; i++)
    for(long j = 0; j < N; j++) C[i * M + j] *= beta;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < N; i++)
    for(long j = 0; j < N; j++)
      for(size_t k = 0; k < M; k++) C[i * N + j] += alpha * A[i * M + k] * A[j * M + k];
}

template <class T>
class Polybench_Syrk {
public:
  Polybench_Syrk(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), opt(poly::options(args, prec)) {
    alpha = opt.has_alpha ? T(opt.alpha) : T(123);
    beta = opt.has_beta ? T(opt.beta) : T(14512);
  }

  void setup() {
    A.resize(size * size);
    C.resize(size * size);
    make_inputs(A.data(), C.data());
    A_buffer.initialize(args.device_queue, A.data(), size * size);
    C_buffer.initialize(args.device_queue, C.data(), size * size);
  }

  void run(std::vector<gb::Event>& events) {
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) {
        poly::host_gemm_body<T>(size, true, alpha, A_buffer.get(), A_buffer.get(), beta, C_buffer.get());
        return;
      }
      const int64_t n = int64_t(size);
      if constexpr(std::is_same<T, float>::value)
        gb::check(gbpoly_syrk_f32(h.ctx(), opt.precision, n, n, alpha, A_buffer.get(), n, beta, C_buffer.get(), n),
            "syrk");
      else
        gb::check(gbpoly_syrk_f64(h.ctx(), n, n, alpha, A_buffer.get(), n, beta, C_buffer.get(), n), "syrk");
    }));
  }

  bool verify(VerificationSetting&) {
    const size_t nn = size * size;
    const T* C_dev = C_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto C_cpu = poly::memo<T>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<T> a(nn), c(nn);
        make_inputs(a.data(), c.data());
        syrk(a.data(), c.data(), size, alpha, beta);
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

  std::string getBenchmarkName(const BenchmarkArgs&) const { return poly::variant_name<T>("Polybench_Syrk", opt); }

  // The reference computes the full square: 2*N^3 operations.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {2.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void make_inputs(T* a, T* c) const {
    if(opt.init == poly::Init::Polybench) {
      init_arrays(a, c, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(c, size * size, opt.init, opt.seed, 2);
    }
  }

  std::vector<double> fp64_reference() const {
    const size_t nn = size * size;
    std::vector<T> a(nn), c(nn);
    make_inputs(a.data(), c.data());
    if(args.device_queue.is_host()) {
      std::vector<double> r(c.begin(), c.end());
      poly::host_gemm_f64(size, false, true, double(alpha), a.data(), a.data(), double(beta), r);
      return r;
    }
    poly::Fp64Device d(args.device_queue, size);
    double *dA = d.upload(a.data()), *dC = d.upload(c.data());
    d.gemm(GBPOLY_OP_N, GBPOLY_OP_T, double(alpha), dA, dA, double(beta), dC);
    return d.download(dC);
  }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  T alpha, beta;
  std::vector<T> A, C;
  PrefetchedBuffer<T, 2> A_buffer, C_buffer;
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
  for(auto p : forms) app.run<Polybench_Syrk<float>>(p);
  if constexpr(SYCL_BENCH_HAS_FP64_SUPPORT) app.run<Polybench_Syrk<double>>();
  return 0;
}
