// MatmulChain: R = (A*B)*(C*D) over N x N matrices (--size), through two
// intermediate products P = A*B and Q = C*D.
// Drop-in for sycl-bench runtime/matmulchain.cpp: same name, identity
// inputs, run() without per-command events, exact-equality verification and
// CSV columns; each product is a libgbpoly contraction writing its output
// (beta = 0, the reference's discard_write).
//
// Accumulator type: the reference kernel (matmulchain.cpp:21) declares its
// running sum `auto sum = 0`, an int, so each product a*b is added to an int
// and truncated toward zero.  On its only inputs, identity matrices, every
// product and sum is 0 or 1 and the int and float sums are equal; the
// contractions here accumulate in float (or in the selected precision form).
//
// Extra options (the reference has none for this benchmark):
//   --precision=...      contraction form(s), as for the PolyBench benchmarks
//   --init=uniform|normal, --seed=   seeded inputs instead of identities; the
//                        result is then checked with the PolyBench comparator
//                        against a host FP32 chain (exact equality is only
//                        meaningful on identities)
//   --graph              the three products as one captured CUDA graph
//   --grouped            P and Q, which are independent, as one grouped launch
//   --verification-oracle, --error-report   as for the PolyBench benchmarks
#include <cstdio>
#include <string>
#include <vector>

#include "polybench_common.h"

template <class T>
class MatmulChain {
public:
  MatmulChain(const BenchmarkArgs& args, gbpoly_precision prec = GBPOLY_PREC_FP32)
      : args(args), mat_size(args.problem_size), opt(poly::options(args, prec)),
        use_graph(args.cli.isFlagSet("--graph") && !args.device_queue.is_host()),
        use_grouped(args.cli.isFlagSet("--grouped") && !args.device_queue.is_host()) {}

  ~MatmulChain() {
    gbpoly_ctx* ctx = args.device_queue.valid() ? args.device_queue.ctx() : nullptr;
    if(graph) gbpoly_graph_destroy(ctx, graph);
    if(grouped) gbpoly_grouped_destroy(ctx, grouped);
  }

  // matmulchain.cpp:56-79
  void setup() {
    const size_t nn = mat_size * mat_size;
    for(auto* v : {&mat_a, &mat_b, &mat_c, &mat_d, &mat_res}) v->assign(nn, T(0));
    make_inputs(mat_a.data(), mat_b.data(), mat_c.data(), mat_d.data());
    mat_a_buf.initialize(args.device_queue, mat_a.data(), nn);
    mat_b_buf.initialize(args.device_queue, mat_b.data(), nn);
    mat_c_buf.initialize(args.device_queue, mat_c.data(), nn);
    mat_d_buf.initialize(args.device_queue, mat_d.data(), nn);
    mat_res_buf.initialize(args.device_queue, mat_res.data(), nn);
    mat_p_buf.initialize(args.device_queue, nn);
    mat_q_buf.initialize(args.device_queue, nn);
    if(use_grouped) plan_grouped();
    if(use_graph) capture_chain();
  }

  // matmulchain.cpp:81-85: three products, no per-command events
  void run() {
    if(use_graph) {
      gb::check(gbpoly_graph_launch(args.device_queue.ctx(), graph), "graph launch");
      return;
    }
    gb::Handler h(args.device_queue);
    chain(h);
  }

  std::string getBenchmarkName(const BenchmarkArgs&) const {
    return poly::variant_name<T>("MatmulChain", opt) + (use_grouped ? "_grouped" : "") + (use_graph ? "_graph" : "");
  }

  // matmulchain.cpp:89-110 on identities: every element equal to the
  // identity's, first mismatch reported on stderr.
  bool verify(VerificationSetting&) {
    const T* res = mat_res_buf.get_host_access();
    const size_t nn = mat_size * mat_size;
    const std::string name = getBenchmarkName(args);
    bool ok = true;
    if(opt.init == poly::Init::Polybench && !opt.fp64_oracle) {
      for(size_t i = 0; i < mat_size && ok; ++i) {
        for(size_t j = 0; j < mat_size; ++j) {
          const T kernel_value = res[i * mat_size + j];
          const T host_value = i == j;
          if(kernel_value != host_value) {
            fprintf(stderr, "VERIFICATION FAILED for element %ld,%ld: %f != %f\n", long(i), long(j),
                double(kernel_value), double(host_value));
            ok = false;
            break;
          }
        }
      }
    } else if(!opt.fp64_oracle) {
      auto ref = poly::memo<T>(poly::memo_key(name, mat_size, opt, "host"), [&] { return host_chain(); });
      ok = poly::compare(ref->data(), res, nn);
    }
    if(opt.fp64_oracle || !opt.error_report.empty()) {
      auto ref = poly::memo<double>(poly::memo_key(name, mat_size, opt, "fp64"), [&] { return fp64_chain(); });
      if(opt.fp64_oracle) ok = poly::compare(ref->data(), res, nn);
      poly::append_error_report(opt, name, mat_size, args.device_queue.device_name(),
          poly::error_norms(res, ref->data(), nn), ok);
    }
    return ok;
  }

  // Not in the reference (it reports no throughput for this benchmark): 3
  // products of 2 N^3 FLOPs.
  static ThroughputMetric getThroughputMetric(const BenchmarkArgs& args) {
    const double n = double(args.problem_size);
    return {6.0 * n * n * n / double(1ull << 30), std::is_same<T, double>::value ? "DP GFLOP" : "SP GFLOP"};
  }

private:
  void chain(gb::Handler& h) {
    if(use_grouped) {
      gb::check(gbpoly_grouped_run(h.ctx(), grouped), "grouped run");
    } else {
      multiply(h, mat_a_buf.get(), mat_b_buf.get(), mat_p_buf.get());  // P = A.B
      multiply(h, mat_c_buf.get(), mat_d_buf.get(), mat_q_buf.get());  // Q = C.D
    }
    multiply(h, mat_p_buf.get(), mat_q_buf.get(), mat_res_buf.get());  // R = P.Q
  }

  // matmulchain.cpp:11-30
  void multiply(gb::Handler& h, const T* a, const T* b, T* c) {
    if(h.on_host()) {
      poly::host_gemm_body<T>(mat_size, false, T(1), a, b, T(0), c);
      return;
    }
    const int64_t n = int64_t(mat_size);
    if constexpr(std::is_same<T, float>::value)
      gb::check(gbpoly_gemm_f32(h.ctx(), opt.precision, GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.f, a, n, b, n, 0.f, c, n),
          "gemm");
    else
      gb::check(gbpoly_gemm_f64(h.ctx(), GBPOLY_OP_N, GBPOLY_OP_N, n, n, n, 1.0, a, n, b, n, 0.0, c, n), "gemm");
  }

  // --grouped: P and Q as one plan (untimed, in setup)
  void plan_grouped() {
    const int64_t n = int64_t(mat_size);
    gbpoly_gemm_desc d[2] = {};
    const T* ops[2][2] = {{mat_a_buf.get(), mat_b_buf.get()}, {mat_c_buf.get(), mat_d_buf.get()}};
    T* outs[2] = {mat_p_buf.get(), mat_q_buf.get()};
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

  // --graph: record the chain into one CUDA graph (untimed, in setup)
  void capture_chain() {
    gbpoly_ctx* ctx = args.device_queue.ctx();
    size_t ws = 0;
    const int64_t n = int64_t(mat_size);
    gb::check(gbpoly_workspace_query(opt.precision, n, n, n, 0, &ws), "workspace query");
    gb::check(gbpoly_workspace_reserve(ctx, ws), "workspace reserve");
    gb::Handler h(args.device_queue);
    gb::check(gbpoly_graph_begin(ctx), "graph begin");
    chain(h);
    gb::check(gbpoly_graph_end(ctx, &graph), "graph end");
  }

  void make_inputs(T* a, T* b, T* c, T* d) const {
    const size_t nn = mat_size * mat_size;
    // --init=polybench (the default) selects the benchmark's own inputs: identities
    if(opt.init == poly::Init::Polybench) {  // matmulchain.cpp:63-71
      for(size_t i = 0; i < mat_size; ++i)
        for(size_t j = 0; j < mat_size; ++j) a[i * mat_size + j] = b[i * mat_size + j] = c[i * mat_size + j] =
            d[i * mat_size + j] = T(i == j);
    } else {
      poly::fill_random(a, nn, opt.init, opt.seed, 0);
      poly::fill_random(b, nn, opt.init, opt.seed, 1);
      poly::fill_random(c, nn, opt.init, opt.seed, 2);
      poly::fill_random(d, nn, opt.init, opt.seed, 3);
    }
  }

  // Host FP32 chain, each element walking k in order.
  std::vector<T> host_chain() const {
    const size_t nn = mat_size * mat_size;
    std::vector<T> a(nn), b(nn), c(nn), d(nn), p(nn), q(nn), r(nn);
    make_inputs(a.data(), b.data(), c.data(), d.data());
    host_product(a.data(), b.data(), p.data());
    host_product(c.data(), d.data(), q.data());
    host_product(p.data(), q.data(), r.data());
    return r;
  }

  void host_product(const T* a, const T* b, T* c) const {
    const long n = long(mat_size);
#pragma omp parallel for schedule(static)
    for(long i = 0; i < n; ++i)
      for(long j = 0; j < n; ++j) {
        T sum = 0;
        for(long k = 0; k < n; ++k) sum += a[i * n + k] * b[k * n + j];
        c[i * n + j] = sum;
      }
  }

  std::vector<double> fp64_chain() const {
    const size_t nn = mat_size * mat_size;
    std::vector<T> a(nn), b(nn), c(nn), d(nn);
    make_inputs(a.data(), b.data(), c.data(), d.data());
    if(args.device_queue.is_host()) {
      std::vector<double> p(nn, 0.0), q(nn, 0.0), r(nn, 0.0);
      poly::host_gemm_f64(mat_size, false, false, 1.0, a.data(), b.data(), 0.0, p);
      poly::host_gemm_f64(mat_size, false, false, 1.0, c.data(), d.data(), 0.0, q);
      poly::host_gemm_f64(mat_size, false, false, 1.0, p.data(), q.data(), 0.0, r);
      return r;
    }
    poly::Fp64Device dev(args.device_queue, mat_size);
    double *dA = dev.upload(a.data()), *dB = dev.upload(b.data()), *dC = dev.upload(c.data());
    double *dD = dev.upload(d.data()), *dP = dev.zeros(), *dQ = dev.zeros(), *dR = dev.zeros();
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dA, dB, 0.0, dP);
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dC, dD, 0.0, dQ);
    dev.gemm(GBPOLY_OP_N, GBPOLY_OP_N, 1.0, dP, dQ, 0.0, dR);
    return dev.download(dR);
  }

  BenchmarkArgs args;
  size_t mat_size;
  poly::Options opt;
  bool use_graph, use_grouped;
  gbpoly_graph* graph = nullptr;
  gbpoly_grouped* grouped = nullptr;
  std::vector<T> mat_a, mat_b, mat_c, mat_d, mat_res;
  PrefetchedBuffer<T, 2> mat_a_buf, mat_b_buf, mat_c_buf, mat_d_buf, mat_res_buf, mat_p_buf, mat_q_buf;
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
  // matmulchain.cpp:113-118: the float chain only
  for(auto p : forms) app.run<MatmulChain<float>>(p);
  return 0;
}
