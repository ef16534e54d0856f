// Polybench_Gesummv: y = ALPHA (A x) + BETA (B x), size x size.
// Drop-in for sycl-bench polybench/gesummv.cpp: same name, initialisation,
// host verification loop and CSV columns.  Its kernel (gesummv.cpp:84-98:
// tmp += A x; y += B x; y = ALPHA tmp + BETA y) is one libgbpoly call,
// gbpoly_gesummv_f32, that reads A and B once each.
#include <string>
#include <vector>

#include "polybench_common.h"

using DATA_TYPE = float;

constexpr DATA_TYPE ALPHA = 1;  // gesummv.cpp:15-16
constexpr DATA_TYPE BETA = 1;

// gesummv.cpp:30-41
void init(DATA_TYPE* A, DATA_TYPE* B, DATA_TYPE* x, size_t size) {
  const auto N = size;
  for(size_t i = 0; i < N; i++) {
    x[i] = 1;
    for(size_t j = 0; j < N; j++) {
      A[i * N + j] = 2;
      B[i * N + j] = 3;
    }
  }
}

// Host oracle, gesummv.cpp:43-56
void gesummv(const DATA_TYPE* A, const DATA_TYPE* B, const DATA_TYPE* x, DATA_TYPE* y, DATA_TYPE* tmp, size_t size) {
  const auto N = size;
  for(size_t i = 0; i < N; i++) {
    tmp[i] = 0;
    y[i] = 0;
    for(size_t j = 0; j < N; j++) {
      tmp[i] = A[i * N + j] * x[j] + tmp[i];
      y[i] = B[i * N + j] * x[j] + y[i];
    }
    y[i] = ALPHA * tmp[i] + BETA * y[i];
  }
}

class Polybench_Gesummv {
public:
  Polybench_Gesummv(const BenchmarkArgs& args)
      : args(args), size(args.problem_size), opt(poly::options(args, GBPOLY_PREC_FP32)) {}

  void setup() {
    A.assign(size * size, 0.f);
    B.assign(size * size, 0.f);
    x.assign(size, 0.f);
    y.assign(size, 0.f);
    tmp.assign(size, 0.f);
    make_inputs(A.data(), B.data(), x.data());
    A_buffer.initialize(args.device_queue, A.data(), size * size);
    B_buffer.initialize(args.device_queue, B.data(), size * size);
    x_buffer.initialize(args.device_queue, x.data(), size);
    y_buffer.initialize(args.device_queue, y.data(), size);
    tmp_buffer.initialize(args.device_queue, tmp.data(), size);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {  // Gesummv
      if(h.on_host()) return host_body();
      gb::check(gbpoly_gesummv_f32(h.ctx(), n, n, ALPHA, A_buffer.get(), n, B_buffer.get(), n, x_buffer.get(), BETA,
                    tmp_buffer.get(), y_buffer.get()),
          "gesummv");
    }));
  }

  // gesummv.cpp:100-117
  bool verify(VerificationSetting&) {
    const DATA_TYPE* y_dev = y_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
      std::vector<DATA_TYPE> a(size * size), b(size * size), xv(size), yc(size), tc(size);
      make_inputs(a.data(), b.data(), xv.data());
      gesummv(a.data(), b.data(), xv.data(), yc.data(), tc.data(), size);
      return yc;
    });
    bool ok = true;
    for(size_t i = 0; i < size && ok; i++)
      if(percentDiff((*ref)[i], y_dev[i]) > poly::kErrorThreshold) ok = false;
    if(!opt.error_report.empty()) {
      auto r64 = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] {
        std::vector<DATA_TYPE> a(size * size), b(size * size), xv(size);
        make_inputs(a.data(), b.data(), xv.data());
        std::vector<double> out(size);
        for(size_t i = 0; i < size; i++) {
          double t = 0, u = 0;
          for(size_t j = 0; j < size; j++) {
            t += double(a[i * size + j]) * double(xv[j]);
            u += double(b[i * size + j]) * double(xv[j]);
          }
          out[i] = double(ALPHA) * t + double(BETA) * u;
        }
        return out;
      });
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(y_dev, r64->data(), size), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<DATA_TYPE>("Polybench_Gesummv", opt);
  }

  // Not in the reference: the matrix bytes read (GiB), A and B once each.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {2.0 * n * n * 4.0 / double(1ull << 30), "GiB"};
  }

private:
  void make_inputs(DATA_TYPE* a, DATA_TYPE* b, DATA_TYPE* xv) const {
    if(opt.init == poly::Init::Polybench) {
      init(a, b, xv, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(b, size * size, opt.init, opt.seed, 1);
      poly::fill_random(xv, size, opt.init, opt.seed, 2);
    }
  }

  // --device=cpu: the reference kernel body (gesummv.cpp:89-97) on the host cores
  void host_body() {
    const float *a = A_buffer.get(), *b = B_buffer.get(), *xv = x_buffer.get();
    float *t = tmp_buffer.get(), *yv = y_buffer.get();
    poly::host_gesummv_body(size, ALPHA, BETA, a, b, xv, t, yv);
  }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  std::vector<DATA_TYPE> A, B, x, y, tmp;
  PrefetchedBuffer<DATA_TYPE, 2> A_buffer, B_buffer;
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
  app.run<Polybench_Gesummv>();  // gesummv.cpp:140-144
  return 0;
}
