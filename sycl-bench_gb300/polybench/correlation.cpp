// Polybench_Correlation: symmat = X^T X of the standardised data matrix,
// with a unit diagonal.
// Drop-in for sycl-bench polybench/correlation.cpp: same name, (size + 1)^2
// arrays used from index 1, initialisation (including its row stride of
// size, correlation.cpp:23-33), host verification loop and CSV columns.  The
// reference's five kernels become five libgbpoly calls:
//   CorrelationMean   (correlation.cpp:111-124)  gbpoly_column_mean_f32
//   CorrelationStd    (correlation.cpp:126-142)  gbpoly_column_stddev_f32
//   CorrelationReduce (correlation.cpp:144-156)  gbpoly_center_columns_f32 into a
//       packed copy with 16-byte-aligned rows (the reference standardises in
//       place; its data buffer is never read back)
//   CorrelationCorr   (correlation.cpp:158-178)  gbpoly_gemm_f32(op_a = T,
//       op_b = N, A == B), the symmetric contraction; its diagonal is then
//   Correlation5      (correlation.cpp:180-186)  set to 1 by gbpoly_set_diagonal_f32
// The reference divides by the double constants FLOAT_N and sqrt(FLOAT_N) in
// CorrelationStd and CorrelationReduce; the device passes use their float
// roundings (each quotient moves by at most one unit in the last place).
// With a split precision form, CorrelationReduce launches nothing and
// CorrelationCorr is gbpoly_covariance_f32, whose split pass centres and
// scales each element as it splits it (same bits, one pass fewer).
#include <cmath>
#include <string>
#include <vector>

#include "polybench_common.h"

#define FLOAT_N 3214212.01
#define EPS 0.005

using DATA_TYPE = float;

// correlation.cpp:23-33, including its row stride of N (not N + 1)
void init_arrays(DATA_TYPE* data, size_t size) {
  const auto M = size;
  const auto N = size;
  for(size_t i = 0; i <= M; i++)
    for(size_t j = 0; j <= N; j++) data[i * N + j] = ((DATA_TYPE)i * j) / (M + 1);
}

// Host oracle, correlation.cpp:35-87 (sequential sums; OpenMP over j1 only).
void correlation(DATA_TYPE* data, DATA_TYPE* mean, DATA_TYPE* stddev, DATA_TYPE* symmat, size_t size) {
  const long M = long(size), N = long(size);
  for(long j = 1; j <= M; j++) {
    mean[j] = 0.0;
    for(long i = 1; i <= N; i++) mean[j] += data[i * (M + 1) + j];
    mean[j] /= (DATA_TYPE)FLOAT_N;
  }
  for(long j = 1; j <= M; j++) {
    stddev[j] = 0.0;
    for(long i = 1; i <= N; i++)
      stddev[j] += (data[i * (M + 1) + j] - mean[j]) * (data[i * (M + 1) + j] - mean[j]);
    stddev[j] /= FLOAT_N;
    stddev[j] = std::sqrt(double(stddev[j]));
    stddev[j] = stddev[j] <= EPS ? 1.0 : stddev[j];
  }
  for(long i = 1; i <= N; i++)
    for(long j = 1; j <= M; j++) {
      data[i * (M + 1) + j] -= mean[j];
      data[i * (M + 1) + j] /= std::sqrt(FLOAT_N);
      data[i * (M + 1) + j] /= stddev[j];
    }
#pragma omp parallel for schedule(dynamic, 4)
  for(long j1 = 1; j1 <= M - 1; j1++) {
    symmat[j1 * (M + 1) + j1] = 1.0;
    for(long j2 = j1 + 1; j2 <= M; j2++) {
      symmat[j1 * (M + 1) + j2] = 0.0;
      for(long i = 1; i <= N; i++) symmat[j1 * (M + 1) + j2] += (data[i * (M + 1) + j1] * data[i * (M + 1) + j2]);
      symmat[j2 * (M + 1) + j1] = symmat[j1 * (M + 1) + j2];
    }
  }
  symmat[M * (M + 1) + M] = 1.0;
}

class Polybench_Correlation {
public:
  Polybench_Correlation(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), size(args.problem_size), ld(size + 1), ldp((size + 31) / 32 * 32),
        opt(poly::options(args, prec)) {}

  void setup() {
    data.assign(ld * ld, 0.f);
    mean.assign(ld, 0.f);
    stddev.assign(ld, 0.f);
    symmat.assign(ld * ld, 0.f);
    make_inputs(data.data());
    data_buffer.initialize(args.device_queue, data.data(), ld * ld);
    mean_buffer.initialize(args.device_queue, mean.data(), ld);
    stddev_buffer.initialize(args.device_queue, stddev.data(), ld);
    symmat_buffer.initialize(args.device_queue, symmat.data(), ld * ld);
    if(!args.device_queue.is_host()) centered_buffer.initialize(args.device_queue, size * ldp);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    float* X = data_buffer.get() + ld + 1;  // element (1, 1)
    float* S = symmat_buffer.get() + ld + 1;
    float* mu = mean_buffer.get() + 1;
    float* sd = stddev_buffer.get() + 1;
    // CorrelationMean
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_mean(X, mu);
      gb::check(gbpoly_column_mean_f32(h.ctx(), n, n, X, int64_t(ld), (DATA_TYPE)FLOAT_N, mu), "column mean");
    }));
    // CorrelationStd
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_std(X, mu, sd);
      gb::check(gbpoly_column_stddev_f32(h.ctx(), n, n, X, int64_t(ld), mu, float(FLOAT_N), float(EPS), sd),
          "column stddev");
    }));
    const bool fused = poly::centres_in_split(opt.precision);
    // CorrelationReduce
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_reduce(X, mu, sd);
      if(fused) return;  // centred and scaled in the contraction's split pass
      gb::check(gbpoly_center_columns_f32(h.ctx(), n, n, X, int64_t(ld), mu, sd, float(std::sqrt(FLOAT_N)),
                    centered_buffer.get(), int64_t(ldp)),
          "normalize columns");
    }));
    // CorrelationCorr
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) return host_corr(X, S);
      if(fused)
        return gb::check(gbpoly_covariance_f32(h.ctx(), opt.precision, n, n, X, int64_t(ld), mu, sd,
                             float(std::sqrt(FLOAT_N)), S, int64_t(ld)),
            "correlation contraction");
      const float* Y = centered_buffer.get();
      gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_T, GBPOLY_OP_N, n, n, n, 1.f, Y, int64_t(ldp), Y,
                    int64_t(ldp), 0.f, S, int64_t(ld)),
          "correlation contraction");
    }));
    // Correlation5 (with the diagonal CorrelationCorr sets)
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {
      if(h.on_host()) {
        if(size > 0) S[(size - 1) * ld + size - 1] = 1.0;
        return;
      }
      gb::check(gbpoly_set_diagonal_f32(h.ctx(), n, 1.f, S, int64_t(ld)), "set diagonal");
    }));
  }

  // correlation.cpp:189-214: percentDiff over rows and columns 1..size
  bool verify(VerificationSetting&) {
    const DATA_TYPE* sym = symmat_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(!opt.fp64_oracle) {
      auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
        std::vector<DATA_TYPE> d(ld * ld, 0.f), m(ld, 0.f), s(ld, 0.f), sy(ld * ld, 0.f);
        make_inputs(d.data());
        correlation(d.data(), m.data(), s.data(), sy.data(), size);
        return sy;
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
    return poly::variant_name<DATA_TYPE>("Polybench_Correlation", opt);
  }

  // Not in the reference (it reports no throughput for this benchmark): the
  // size (size - 1) / 2 off-diagonal outputs of 2 * size FLOPs each.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {n * n * (n > 0 ? n - 1 : 0) / double(1ull << 30), "SP GFLOP"};
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

  // --device=cpu: the reference kernel bodies (correlation.cpp:115-185) on the host cores
  void host_mean(const float* X, float* mu) const {
    poly::host_column_sums(size, size, ld, X, mu, [](float x, size_t) { return x; });
    for(size_t j = 0; j < size; ++j) mu[j] /= ((DATA_TYPE)FLOAT_N);
  }
  void host_std(const float* X, const float* mu, float* sd) const {
    poly::host_column_sums(size, size, ld, X, sd, [mu](float x, size_t j) { return (x - mu[j]) * (x - mu[j]); });
    for(size_t j = 0; j < size; ++j) {
      sd[j] /= FLOAT_N;
      sd[j] = std::sqrt(sd[j]);
      sd[j] = sd[j] <= EPS ? 1.0 : sd[j];
    }
  }
  void host_reduce(float* X, const float* mu, const float* sd) const {
#pragma omp parallel for schedule(static)
    for(long i = 0; i < long(size); ++i)
      for(size_t j = 0; j < size; ++j) {
        X[i * ld + j] -= mu[j];
        X[i * ld + j] /= std::sqrt(FLOAT_N);
        X[i * ld + j] /= sd[j];
      }
  }
  void host_corr(const float* X, float* S) const {
    for(size_t j = 0; j < size; j++) S[j * ld + j] = 1.0;
    poly::host_xtx_upper(size, ld, X, S, 1);
  }

  // FP64 result of the same program: statistics, standardisation and the
  // contraction in double with the program's constants; unit diagonal.
  std::vector<double> fp64_reference() const {
    std::vector<DATA_TYPE> d(ld * ld, 0.f);
    make_inputs(d.data());
    std::vector<double> x(size * size), mu(size, 0.0), sd(size, 0.0);
    for(size_t j = 0; j < size; ++j) {
      for(size_t i = 0; i < size; ++i) mu[j] += double(d[(i + 1) * ld + j + 1]);
      mu[j] /= double((DATA_TYPE)FLOAT_N);
      for(size_t i = 0; i < size; ++i) {
        const double c = double(d[(i + 1) * ld + j + 1]) - mu[j];
        sd[j] += c * c;
      }
      sd[j] = std::sqrt(sd[j] / FLOAT_N);
      if(sd[j] <= EPS) sd[j] = 1.0;
    }
    for(size_t i = 0; i < size; ++i)
      for(size_t j = 0; j < size; ++j)
        x[i * size + j] = (double(d[(i + 1) * ld + j + 1]) - mu[j]) / std::sqrt(FLOAT_N) / sd[j];
    std::vector<double> s;
    if(args.device_queue.is_host()) {
      s.assign(size * size, 0.0);
      poly::host_gemm_f64(size, true, false, 1.0, x.data(), x.data(), 0.0, s);
    } else {
      poly::Fp64Device dev(args.device_queue, size);
      double *dX = dev.upload(x.data()), *dS = dev.zeros();
      dev.gemm(GBPOLY_OP_T, GBPOLY_OP_N, 1.0, dX, dX, 0.0, dS);
      s = dev.download(dS);
    }
    for(size_t j = 0; j < size; ++j) s[j * size + j] = 1.0;
    return s;
  }

  BenchmarkArgs args;
  const size_t size, ld, ldp;
  poly::Options opt;
  std::vector<DATA_TYPE> data, mean, stddev, symmat;
  PrefetchedBuffer<DATA_TYPE, 2> data_buffer, symmat_buffer, centered_buffer;
  PrefetchedBuffer<DATA_TYPE, 1> mean_buffer, stddev_buffer;
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
  for(auto p : forms) app.run<Polybench_Correlation>(p);  // correlation.cpp:230-234
  return 0;
}
