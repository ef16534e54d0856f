// Polybench_Syr2k: C = beta*C + alpha*(A*B^T + B*A^T) over the full N x N
// square (N = M = --size), alpha = beta = 1.  Drop-in for sycl-bench
// polybench/syr2k.cpp: same name, initialisation, host verification loop and
// CSV columns; the device kernel accumulates both products in one pass.
#include <string>
#include <vector>

#include "polybench_common.h"

// syr2k.cpp:18-32
template <class T>
void init_arrays(T* A, T* B, T* C, size_t size) {
  const auto N = size, M = size;
  for(size_t i = 0; i < N; i++) {
    for(size_t j = 0; j < N; j++) C[i * N + j] = ((T)i * j + 2) / N;
    for(size_t j = 0; j < M; j++) {
      A[i * N + j] = ((T)i * j) / N;
      B[i * N + j] = ((T)i * j + 1) / N;
    }
  }
}

// Host oracle, syr2k.cpp:34-52: two separate accumulations per k.
template <class T>
void syr2k(const T* A, const T* B, T* C, size_t size, T alpha, T beta) {
  const long N = long(size);
  const size_t M = size;
  for(long i = 0; i < N; i++)
    for(long j = 0; j < N; j++) C[i * N + j] *= beta;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < N; i++)
    for(long j = 0; j < N; j++)
      for(size_t k = 0; k < M; k++) {
        C[i * N + j] += alpha * A[i * M + k] * B[j * M + k];
        C[i * N + j] += alpha * B[i * M + k] * A[j * M + k];
      }
}

template <class T>
class Polybench_Syr2k {
public:
  Polybench_Syr2k(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), opt(poly::options(args, prec)) {
    alpha = opt.has_alpha ? T(opt.alpha) : T(1);
    beta = opt.has_beta ? T(opt.beta) : T(1);
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
        poly::host_syr2k_body<T>(size, alpha, A_buffer.get(), B_buffer.get(), beta, C_buffer.get());
        return;
      }
      const int64_t n = int64_t(size);
      if constexpr(std::is_same<T, float>::value)
        gb::check(gbpoly_syr2k_f32(h.ctx(), opt.precision, n, n, alpha, A_buffer.get(), n, B_buffer.get(), n, beta,
                      C_buffer.get(), n),
            "syr2k");
      else
        gb::check(gbpoly_syr2k_f64(h.ctx(), n, n, alpha, A_buffer.get(), n, B_buffer.get(), n, beta, C_buffer.get(), n),
            "syr2k");
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
        syr2k(a.data(), b.data(), c.data(), size, alpha, beta);
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

  std::string getBenchmarkName(const BenchmarkArgs&) const { return poly::variant_name<T>("Polybench_Syr2k", opt); }

  // Full square, two products: 4*N^3 operations.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {4.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void make_inputs(T* a, T* b, T* c) const {
    if(opt.init == poly::Init::Polybench) {
      init_arrays(a, b, c, size);
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
      poly::host_gemm_f64(size, false, true, double(alpha), a.data(), b.data(), double(beta), r);
      poly::host_gemm_f64(size, false, true, double(alpha), b.data(), a.data(), 1.0, r);
      return r;
    }
    poly::Fp64Device d(args.device_queue, size);
    double *dA = d.upload(a.data()), *dB = d.upload(b.data()), *dC = d.upload(c.data());
    d.gemm(GBPOLY_OP_N, GBPOLY_OP_T, double(alpha), dA, dB, double(beta), dC);
    d.gemm(GBPOLY_OP_N, GBPOLY_OP_T, double(alpha), dB, dA, 1.0, dC);
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
  for(auto p : forms) app.run<Polybench_Syr2k<float>>(p);
  if constexpr(SYCL_BENCH_HAS_FP64_SUPPORT) app.run<Polybench_Syr2k<double>>();
  return 0;
}
