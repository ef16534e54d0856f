// Polybench_Bicg: s = A^T r and q = A p, size x size.
// Drop-in for sycl-bench polybench/bicg.cpp: same name, initialisation, host
// verification loop and CSV columns.  Its two kernels, Bicg1 (s += A^T r,
// bicg.cpp:77-88) and Bicg2 (q += A p, bicg.cpp:90-100), read the same A;
// here they are one libgbpoly call (gbpoly_gemv_pair_f32) that reads A once,
// recorded as one command.
#include <cmath>
#include <string>
#include <vector>

#include "polybench_common.h"

#ifndef M_PI
#define M_PI 3.14159
#endif

using DATA_TYPE = float;

// bicg.cpp:20-35
void init_array(DATA_TYPE* A, DATA_TYPE* p, DATA_TYPE* r, size_t size) {
  const auto NX = size;
  const auto NY = size;
  for(size_t i = 0; i < NX; i++) {
    r[i] = i * M_PI;
    for(size_t j = 0; j < NY; j++) A[i * NY + j] = ((DATA_TYPE)i * j) / NX;
  }
  for(size_t i = 0; i < NY; i++) p[i] = i * M_PI;
}

// Host oracle, bicg.cpp:37-48
void bicg_cpu(const DATA_TYPE* A, const DATA_TYPE* r, DATA_TYPE* s, const DATA_TYPE* p, DATA_TYPE* q, size_t size) {
  const auto NX = size;
  const auto NY = size;
  for(size_t i = 0; i < NX; i++)
    for(size_t j = 0; j < NY; j++) {
      s[j] += r[i] * A[i * NY + j];
      q[i] += A[i * NY + j] * p[j];
    }
}

class Polybench_Bicg {
public:
  Polybench_Bicg(const BenchmarkArgs& args) : args(args), size(args.problem_size), opt(poly::options(args, GBPOLY_PREC_FP32)) {}

  void setup() {
    A.assign(size * size, 0.f);
    r.assign(size, 0.f);
    s.assign(size, 0.f);
    p.assign(size, 0.f);
    q.assign(size, 0.f);
    make_inputs(A.data(), p.data(), r.data());
    A_buffer.initialize(args.device_queue, A.data(), size * size);
    r_buffer.initialize(args.device_queue, r.data(), size);
    s_buffer.initialize(args.device_queue, s.data(), size);
    p_buffer.initialize(args.device_queue, p.data(), size);
    q_buffer.initialize(args.device_queue, q.data(), size);
  }

  void run(std::vector<gb::Event>& events) {
    const int64_t n = int64_t(size);
    events.push_back(args.device_queue.submit([&](gb::Handler& h) {  // Bicg1 + Bicg2
      if(h.on_host()) {
        host_cols(A_buffer.get(), r_buffer.get(), s_buffer.get());
        host_rows(A_buffer.get(), p_buffer.get(), q_buffer.get());
        return;
      }
      const gbpoly_gemv_term terms[2] = {{GBPOLY_OP_T, 1.f, 1.f, r_buffer.get(), s_buffer.get()},
          {GBPOLY_OP_N, 1.f, 1.f, p_buffer.get(), q_buffer.get()}};
      gb::check(gbpoly_gemv_pair_f32(h.ctx(), n, n, A_buffer.get(), n, terms, 2), "gemv pair");
    }));
  }

  // bicg.cpp:102-124: s and q element by element
  bool verify(VerificationSetting&) {
    const DATA_TYPE* s_dev = s_buffer.get_host_access();
    std::vector<DATA_TYPE> s_copy(s_dev, s_dev + size);
    const DATA_TYPE* q_dev = q_buffer.get_host_access();
    const std::string name = getBenchmarkName(args);
    auto ref = poly::memo<DATA_TYPE>(poly::memo_key(name, size, opt, "host"), [&] {
      std::vector<DATA_TYPE> a(size * size), pv(size), rv(size), sc(size), qc(size);
      make_inputs(a.data(), pv.data(), rv.data());
      bicg_cpu(a.data(), rv.data(), sc.data(), pv.data(), qc.data(), size);
      sc.insert(sc.end(), qc.begin(), qc.end());
      return sc;
    });
    bool ok = true;
    for(size_t i = 0; i < size && ok; i++) {
      if(percentDiff((*ref)[i], s_copy[i]) > poly::kErrorThreshold) ok = false;
      if(percentDiff((*ref)[size + i], q_dev[i]) > poly::kErrorThreshold) ok = false;
    }
    if(!opt.error_report.empty()) {
      auto r64 = poly::memo<double>(poly::memo_key(name, size, opt, "fp64"), [&] {
        std::vector<DATA_TYPE> a(size * size), pv(size), rv(size);
        make_inputs(a.data(), pv.data(), rv.data());
        std::vector<double> out(2 * size, 0.0);
        for(size_t i = 0; i < size; i++)
          for(size_t j = 0; j < size; j++) {
            out[j] += double(rv[i]) * double(a[i * size + j]);
            out[size + i] += double(a[i * size + j]) * double(pv[j]);
          }
        return out;
      });
      std::vector<DATA_TYPE> got(s_copy);
      got.insert(got.end(), q_dev, q_dev + size);
      poly::append_error_report(opt, name, size, args.device_queue.device_name(),
          poly::error_norms(got.data(), r64->data(), 2 * size), ok);
    }
    return ok;
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const { return poly::variant_name<DATA_TYPE>("Polybench_Bicg", opt); }

  // Not in the reference: the matrix bytes read (GiB), once for both products.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {n * n * 4.0 / double(1ull << 30), "GiB"};
  }

private:
  void make_inputs(DATA_TYPE* a, DATA_TYPE* pv, DATA_TYPE* rv) const {
    if(opt.init == poly::Init::Polybench) {
      init_array(a, pv, rv, size);
    } else {
      poly::fill_random(a, size * size, opt.init, opt.seed, 0);
      poly::fill_random(pv, size, opt.init, opt.seed, 1);
      poly::fill_random(rv, size, opt.init, opt.seed, 2);
    }
  }

  // --device=cpu: the reference kernel bodies (bicg.cpp:82-98) on the host cores
  void host_cols(const float* a, const float* rv, float* sv) const { poly::host_gemv_t_body(size, a, rv, sv); }
  void host_rows(const float* a, const float* pv, float* qv) const { poly::host_gemv_n_body(size, a, pv, qv); }

  BenchmarkArgs args;
  const size_t size;
  poly::Options opt;
  std::vector<DATA_TYPE> A, r, s, p, q;
  PrefetchedBuffer<DATA_TYPE, 2> A_buffer;
  PrefetchedBuffer<DATA_TYPE, 1> r_buffer, s_buffer, p_buffer, q_buffer;
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
  app.run<Polybench_Bicg>();  // bicg.cpp:145-149
  return 0;
}
