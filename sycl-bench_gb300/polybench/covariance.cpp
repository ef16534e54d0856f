// Polybench_Covariance: symmat = X^T X of the column-centred data matrix.
// Drop-in for sycl-bench polybench/covariance.cpp: same name, (size + 1)^2
// arrays used from index 1, initialisation, host verification loop and CSV
// columns.  The reference's three kernels become three libgbpoly calls:
//   CovarianceMean   (covariance.cpp:84-96)   gbpoly_column_mean_f32
//   CovarianceReduce (covariance.cpp:98-106)  gbpoly_center_columns_f32, which
//       writes the centred block into a packed copy (16-byte-aligned rows) that
//       feeds the contraction; the reference centres in place, and its data
//       buffer is never read back, so nothing observable differs
//   CovarianceCovar  (covariance.cpp:108-126) gbpoly_gemm_f32(op_a = T,
//       op_b = N, A == B): the symmetric contraction, lower triangle of tiles
//       computed and mirrored; the reference computes j2 >= j1 and mirrors.
// With a split precision form, CovarianceReduce launches nothing and
// CovarianceCovar is gbpoly_covariance_f32, whose split pass centres each
// element as it splits it (same bits, one pass over the data fewer).
#include <cmath>
#include <string>
#include <vector>

#include "polybench_common.h"

using DATA_TYPE = float;

constexpr DATA_TYPE float_n = 3214212.01;  // covariance.cpp:18 (a float constant)

// covariance.cpp:20-29: rows and columns 0..size-1 of the (size+1)^2 array
void init_arrays(DATA_TYPE* data, size_t size) {
  const auto M = size;
  const auto N = size;
  for(size_t i = 0; i < M; i++)
    for(size_t j = 0; j < N; j++) data[i * (N + 1) + j] = ((DATA_TYPE)i * j) / M;
}

// Host oracle, covariance.cpp:31-60 (sequential sums; OpenMP over j1 only).
void covariance(DATA_TYPE* data, DATA_TYPE* symmat, DATA_TYPE* mean, size_t size) {
  const long M = long(size), N = long(size);
  for(long j = 1; j <= M; j++) {
    mean[j] = 0.0;
    for(long i = 1; i <= N; i++) mean[j] += data[i * (M + 1) + j];
    mean[j] /= float_n;
  }
  for(long i = 1; i <= N; i++)
    for(long j = 1; j <= M; j++) data[i * (M + 1) + j] -= mean[j];
#pragma omp parallel for schedule(dynamic, 4)
  for(long j1 = 1; j1 <= M; j1++)
    for(long j2 = j1; j2 <= M; j2++) {
      symmat[j1 * (M + 1) + j2] = 0.0;
      for(long i = 1; i <= N; i++) symmat[j1 * (M + 1) + j2] += data[i * (M + 1) + j1] * data[i * (M + 1) + j2];
      symmat[j2 * (M + 1) + j1] = symmat[j1 * (M + 1) + j2];
    }
}

class Polybench_Covariance {
public:
  Polybench_Covariance(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), ld(size + 1), ldp((size + 31) / 32 * 32),
        opt(poly::options(args, prec)) {}

  void setup() {
    data.assign(ld * ld, 0.f);
    symmat.assign(ld * ld, 0.f);
    mean.assign(ld, 0.f);
    make_inputs(data.data());
    data_buffer.initialize(args.device_queue, data.data(), ld * ld);
    symmat_buffer.initialize(args.device_queue, symmat.data(), ld * ld);
    mean_buffer.initialize(args.device_queue, mean.data(), ld);
    if(!args.device_queue.is_host()) centered_buffer.initialize(args.device_queue, size * ldp);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    float* X = data_buffer.get() + ld + 1;  // element (1, 1)
    float* S = symmat_buffer.get() + ld + 1;
    float* mu = mean_buffer.get() + 1;
    // CovarianceMean
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_mean(X, mu);
      gb::check(gbpoly_column_mean_f32(h.ctx(), n, n, X, int64_t(ld), float_n, mu), "column mean");
    }));
    const bool fused = poly::centres_in_split(opt.precision);
    // CovarianceReduce
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_center(X, mu);
      if(fused) return;  // centred in the contraction's split pass
      gb::check(gbpoly_center_columns_f32(h.ctx(), n, n, X, int64_t(ld), mu, nullptr, 1.f, centered_buffer.get(),
                    int64_t(ldp)),
          "center columns");
    }));
    // CovarianceCovar
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_covar(X, S);
      if(fused)
        return gb::check(gbpoly_covariance_f32(h.ctx(), opt.precision, n, n, X, int64_t(ld), mu, nullptr, 1.f, S,
                             int64_t(ld)),
            "covariance contraction");
      const float* Y = centered_buffer.get();
      gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_T, GBPOLY_OP_N, n, n, n, 1.f, Y, int64_t(ldp), Y,
                    int64_t(ldp), 0.f, S, int64_t(ld)),
          "covariance contraction");
    }));
  }

  // covariance.cpp:129-152: percentDiff over rows and columns 1..size
  bool verify(VerificationSetting&) {
    const DATA_TYPE* sym = symmat_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<DATA_TYPE> d(ld * ld, 0.f), s(ld * ld, 0.f), m(ld, 0.f);
        make_inputs(d.data());
        covariance(d.data(), s.data(), m.data(), size);
        return s;
      });
      ok = interior_compare(ref->data(), sym);
    }
    if(opt.fp64_oracle || !opt.error_report.empty()) {
      auto ref = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] { return fp64_reference(); });
      std::vector<float> got(size * size);
      for(size_t i = 0; i < size; ++i)
        for(size_t j = 0; j < size; ++j) got[i * size + j] = sym[(i + 1) * ld + j + 1];
      if(opt.fp64_oracle) ok = poly::compare(ref->data(), got.data(), size * size);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(got.data(), ref->data(), size * size), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<DATA_TYPE>("Polybench_Covariance", opt);
  }

  // Not in the reference (it reports no throughput for this benchmark): the
  // size (size + 1) / 2 distinct outputs of 2 * size FLOPs each.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {n * n * (n + 1) / double(1ull << 30), "SP GFLOP"};
  }

private:
  template <class R>
  bool interior_compare(const R* ref, const DATA_TYPE* dev) const {
    for(size_t i = 1; i < size + 1; i++)
      for(size_t j = 1; j < size + 1; j++)
        if(percentDiff(ref[i * ld + j], dev[i * ld + j]) > poly::kErrorThreshold) return false;
    return true;
  }

  void make_inputs(DATA_TYPE* d) const {
    if(opt.init == poly::Init::Polybench)
      init_arrays(d, size);
    else
      poly::fill_random(d, ld * ld, opt.init, opt.seed, 0);
  }

  // --device=cpu: the reference kernel bodies (covariance.cpp:89-124) on the host cores
  void host_mean(const float* X, float* mu) const {
    for(size_t j = 0; j < size; ++j) mu[j] = 0;
    poly::host_column_sums(size, size, ld, X, mu, [](float x, size_t) { return x; });
    for(size_t j = 0; j < size; ++j) mu[j] /= float_n;
  }
  void host_center(float* X, const float* mu) const {
#pragma omp parallel for schedule(static)
    for(long i = 0; i < long(size); ++i)
      for(size_t j = 0; j < size; ++j) X[i * ld + j] -= mu[j];
  }
  // The diagonal's 1.0 (covariance.cpp:118) is overwritten by its own sum.
  void host_covar(const float* X, float* S) const { poly::host_xtx_upper(size, ld, X, S, 0); }

  // FP64 result of the same program: means, centring and the contraction in
  // double (the divisor is the float constant the program uses).
  std::vector<double> fp64_reference() const {
    std::vector<DATA_TYPE> d(ld * ld, 0.f);
    make_inputs(d.data());
    std::vector<double> x(size * size), mu(size, 0.0);
    for(size_t j = 0; j < size; ++j) {
      for(size_t i = 0; i < size; ++i) mu[j] += double(d[(i + 1) * ld + j + 1]);
      mu[j] /= double(float_n);
    }
    for(size_t i = 0; i < size; ++i)
      for(size_t j = 0; j < size; ++j) x[i * size + j] = double(d[(i + 1) * ld + j + 1]) - mu[j];
    if(args.device_queue.is_host()) {
      std::vector<double> s(size * size, 0.0);
      poly::host_gemm_f64(size, true, false, 1.0, x.data(), x.data(), 0.0, s);
      return s;
    }
    poly::Fp64Device dev(args.device_queue, size);
    double *dX = dev.upload(x.data()), *dS = dev.zeros();
    dev.gemm(GBPOLY_OP_T, GBPOLY_OP_N, 1.0, dX, dX, 0.0, dS);
    return dev.download(dS);
  }

  BenchmarkArgs args;
  const size_t size, ld, ldp;
  poly::Options opt;
  std::vector<DATA_TYPE> data, symmat, mean;
  PrefetchedBuffer<DATA_TYPE, 2> data_buffer, symmat_buffer, centered_buffer;
  PrefetchedBuffer<DATA_TYPE, 1> mean_buffer;
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
  for(auto p : forms) app.run<Polybench_Covariance>(p);  // covariance.cpp:170-174
  return 0;
}
