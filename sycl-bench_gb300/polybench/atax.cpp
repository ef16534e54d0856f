// Polybench_Atax: y = A^T (A x) through tmp = A x, size x size.
// Drop-in for sycl-bench polybench/atax.cpp: same name, initialisation, host
// verification loop and CSV columns.  Its two kernels, Atax1 (tmp += A x,
// atax.cpp:73-84) and Atax2 (y += A^T tmp, atax.cpp:86-97), are one libgbpoly
// call (gbpoly_atax_f32), recorded as one command: up to 8192 columns one
// kernel reads A from HBM once (a row group's dots, then the same rows again
// from L2 for the column sums); wider matrices take two passes.
#include <cmath>
#include <string>
#include <vector>

#include "polybench_common.h"

#ifndef M_PI
#define M_PI 3.14159
#endif

using DATA_TYPE = float;

// atax.cpp:20-30
void init_array(DATA_TYPE* x, DATA_TYPE* A, size_t size) {
  const auto NX = size;
  const auto NY = size;
  for(size_t i = 0; i < NX; i++) {
    x[i] = i * M_PI;
    for(size_t j = 0; j < NY; j++) A[i * NY + j] = ((DATA_TYPE)i * (j)) / NX;
  }
}

// Host oracle, atax.cpp:32-46 (y accumulated row by row, as written).
void atax_cpu(const DATA_TYPE* A, const DATA_TYPE* x, DATA_TYPE* y, DATA_TYPE* tmp, size_t size) {
  const auto NX = size;
  const auto NY = size;
  for(size_t i = 0; i < NX; i++) {
    for(size_t j = 0; j < NY; j++) tmp[i] += A[i * NY + j] * x[j];
    for(size_t j = 0; j < NY; j++) y[j] += A[i * NY + j] * tmp[i];
  }
}

class Polybench_Atax {
public:
  Polybench_Atax(const BenchmarkArgs& args) : args(args), size(args.problem_size), opt(poly::options(args, GBPOLY_PREC_FP32)) {}

  void setup() {
    A.assign(size * size, 0.f);
    x.assign(size, 0.f);
    y.assign(size, 0.f);
    tmp.assign(size, 0.f);
    make_inputs(x.data(), A.data());
    A_buffer.initialize(args.device_queue, A.data(), size * size);
    x_buffer.initialize(args.device_queue, x.data(), size);
    y_buffer.initialize(args.device_queue, y.data(), size);
    tmp_buffer.initialize(args.device_queue, tmp.data(), size);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {  // Atax1 + Atax2
      if(h.on_host()) {
        host_rows(A_buffer.get(), x_buffer.get(), tmp_buffer.get());
        host_cols(A_buffer.get(), tmp_buffer.get(), y_buffer.get());
        return;
      }
      gb::check(gbpoly_atax_f32(h.ctx(), n, n, A_buffer.get(), n, x_buffer.get(), tmp_buffer.get(), y_buffer.get()),
          "atax");
    }));
  }

  // atax.cpp:100-120
  bool verify(VerificationSetting&) {
    const DATA_TYPE* y_dev = y_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
      std::vector<DATA_TYPE> a(size * size), xv(size), yc(size), tc(size);
      make_inputs(xv.data(), a.data());
      atax_cpu(a.data(), xv.data(), yc.data(), tc.data(), size);
      return yc;
    });
    bool ok = true;
    for(size_t i = 0; i < size && ok; i++)
      if(percentDiff((*ref)[i], y_dev[i]) > poly::kErrorThreshold) ok = false;
    if(!opt.error_report.empty()) {
      auto r64 = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] {
        std::vector<DATA_TYPE> a(size * size), xv(size);
        make_inputs(xv.data(), a.data());
        std::vector<double> t(size, 0.0), yy(size, 0.0);
        for(size_t i = 0; i < size; i++)
          for(size_t j = 0; j < size; j++) t[i] += double(a[i * size + j]) * double(xv[j]);
        for(size_t i = 0; i < size; i++)
          for(size_t j = 0; j < size; j++) yy[j] += double(a[i * size + j]) * t[i];
        return yy;
      });
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(y_dev, r64->data(), size), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const { return poly::variant_name<DATA_TYPE>("Polybench_Atax", opt); }

  // Not in the reference: the matrix bytes one read of A moves (GiB), so the
  // throughput columns read as matrix bandwidth.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {n * n * 4.0 / double(1ull << 30), "GiB"};
  }

private:
  void make_inputs(DATA_TYPE* xv, DATA_TYPE* a) const {
    if(opt.init == poly::Init::Polybench) {
      init_array(xv, a, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(xv, size, opt.init, opt.seed, 1);
    }
  }

  // --device=cpu: the reference kernel bodies (atax.cpp:78-95) on the host cores
  void host_rows(const float* a, const float* xv, float* t) const { poly::host_gemv_n_body(size, a, xv, t); }
  void host_cols(const float* a, const float* t, float* yv) const { poly::host_gemv_t_body(size, a, t, yv); }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  std::vector<DATA_TYPE> A, x, y, tmp;
  PrefetchedBuffer<DATA_TYPE, 2> A_buffer;
  PrefetchedBuffer<DATA_TYPE, 1> x_buffer, y_buffer, tmp_buffer;
};

int main(int argc, char** argv) {
  BenchmarkApp app(argc, argv);
  if(!app.getArgs().device_queue.valid()) return 0;
  try {
    poly::require_fp32_only(app.getArgs());
  } catch(std::exception& e) {
    std::cerr << "Error: " << e.what() << std::endl;
    return 0;
  }
  app.run<Polybench_Atax>();  // atax.cpp:144-148
  return 0;
}
