// Polybench_Mvt: x1 += A y1 and x2 += A y2, size x size.
// Drop-in for sycl-bench polybench/mvt.cpp: same name, initialisation, host
// verification loop and CSV columns.  The reference's second product reads A
// itself (mvt.cpp:36-40 and :92-96, x2[k] += a[k][l] * y2[l]; PolyBench/C's
// mvt uses A^T there), and so does this one.  Its two kernels, Mvt1
// (mvt.cpp:75-86) and Mvt2 (mvt.cpp:88-98), read the same A; here they are
// one libgbpoly call (gbpoly_gemv_pair_f32) that reads A once, recorded as
// one command.
#include <string>
#include <vector>

#include "polybench_common.h"

using DATA_TYPE = float;

// mvt.cpp:16-28
void init_arrays(DATA_TYPE* a, DATA_TYPE* x1, DATA_TYPE* x2, DATA_TYPE* y_1, DATA_TYPE* y_2, size_t size) {
  const auto N = size;
  for(size_t i = 0; i < N; i++) {
    x1[i] = 0.0;
    x2[i] = 0.0;
    y_1[i] = 1.0;
    y_2[i] = 1.0;
    for(size_t j = 0; j < N; j++) a[i * N + j] = (DATA_TYPE)(i + j + 1.0) / N;
  }
}

// Host oracle, mvt.cpp:30-42
void runMvt(const DATA_TYPE* a, DATA_TYPE* x1, DATA_TYPE* x2, const DATA_TYPE* y1, const DATA_TYPE* y2, size_t size) {
  const auto N = size;
  for(size_t i = 0; i < N; i++)
    for(size_t j = 0; j < N; j++) x1[i] = x1[i] + a[i * N + j] * y1[j];
  for(size_t k = 0; k < N; k++)
    for(size_t l = 0; l < N; l++) x2[k] = x2[k] + a[k * N + l] * y2[l];
}

class Polybench_Mvt {
public:
  Polybench_Mvt(const BenchmarkArgs& args) : args(args), size(args.problem_size), opt(poly::options(args, GBPOLY_PREC_FP32)) {}

  void setup() {
    a.assign(size * size, 0.f);
    for(auto* v : {&x1, &x2, &y1, &y2}) v->assign(size, 0.f);
    make_inputs(a.data(), x1.data(), x2.data(), y1.data(), y2.data());
    a_buffer.initialize(args.device_queue, a.data(), size * size);
    x1_buffer.initialize(args.device_queue, x1.data(), size);
    x2_buffer.initialize(args.device_queue, x2.data(), size);
    y1_buffer.initialize(args.device_queue, y1.data(), size);
    y2_buffer.initialize(args.device_queue, y2.data(), size);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {  // Mvt1 + Mvt2
      if(h.on_host()) {
        host_rows(a_buffer.get(), y1_buffer.get(), x1_buffer.get());
        host_rows(a_buffer.get(), y2_buffer.get(), x2_buffer.get());
        return;
      }
      const gbpoly_gemv_term terms[2] = {{GBPOLY_OP_N, 1.f, 1.f, y1_buffer.get(), x1_buffer.get()},
          {GBPOLY_OP_N, 1.f, 1.f, y2_buffer.get(), x2_buffer.get()}};
      gb::check(gbpoly_gemv_pair_f32(h.ctx(), n, n, a_buffer.get(), n, terms, 2), "gemv pair");
    }));
  }

  // mvt.cpp:100-124: x1 and x2 element by element
  bool verify(VerificationSetting&) {
    const DATA_TYPE* x1_dev = x1_buffer.get_host_access();
    std::vector<DATA_TYPE> x1_copy(x1_dev, x1_dev + size);
    const DATA_TYPE* x2_dev = x2_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
      std::vector<DATA_TYPE> av(size * size), a1(size), a2(size), b1(size), b2(size);
      make_inputs(av.data(), a1.data(), a2.data(), b1.data(), b2.data());
      runMvt(av.data(), a1.data(), a2.data(), b1.data(), b2.data(), size);
      a1.insert(a1.end(), a2.begin(), a2.end());
      return a1;
    });
    bool ok = true;
    for(size_t i = 0; i < size && ok; i++) {
      if(percentDiff((*ref)[i], x1_copy[i]) > poly::kErrorThreshold) ok = false;
      if(percentDiff((*ref)[size + i], x2_dev[i]) > poly::kErrorThreshold) ok = false;
    }
    if(!opt.error_report.empty()) {
      auto r64 = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] {
        std::vector<DATA_TYPE> av(size * size), a1(size), a2(size), b1(size), b2(size);
        make_inputs(av.data(), a1.data(), a2.data(), b1.data(), b2.data());
        std::vector<double> out(2 * size);
        for(size_t i = 0; i < size; i++) {
          double s1 = a1[i], s2 = a2[i];
          for(size_t j = 0; j < size; j++) {
            s1 += double(av[i * size + j]) * double(b1[j]);
            s2 += double(av[i * size + j]) * double(b2[j]);
          }
          out[i] = s1;
          out[size + i] = s2;
        }
        return out;
      });
      std::vector<DATA_TYPE> got(x1_copy);
      got.insert(got.end(), x2_dev, x2_dev + size);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(got.data(), r64->data(), 2 * size), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const { return poly::variant_name<DATA_TYPE>("Polybench_Mvt", opt); }

  // Not in the reference: the matrix bytes read (GiB), once for both products.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {n * n * 4.0 / double(1ull << 30), "GiB"};
  }

private:
  void make_inputs(DATA_TYPE* av, DATA_TYPE* a1, DATA_TYPE* a2, DATA_TYPE* b1, DATA_TYPE* b2) const {
    init_arrays(av, a1, a2, b1, b2, size);
    if(opt.init != poly::Init::Polybench) {  // seeded matrix and right-hand sides, zero x1/x2
      poly::fill_random(av, size * size, opt.init, opt.seed, 0);
      poly::fill_random(b1, size, opt.init, opt.seed, 1);
      poly::fill_random(b2, size, opt.init, opt.seed, 2);
    }
  }

  // --device=cpu: the reference kernel bodies (mvt.cpp:80-96) on the host cores
  void host_rows(const float* av, const float* yv, float* xv) const { poly::host_gemv_n_body(size, av, yv, xv); }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  std::vector<DATA_TYPE> a, x1, x2, y1, y2;
  PrefetchedBuffer<DATA_TYPE, 2> a_buffer;
  PrefetchedBuffer<DATA_TYPE, 1> x1_buffer, x2_buffer, y1_buffer, y2_buffer;
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
  app.run<Polybench_Mvt>();  // mvt.cpp:145-149
  return 0;
}
