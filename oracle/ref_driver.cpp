// Driver around one of the reference's own PolyBench sources (TEST
// INFRASTRUCTURE, built by oracle/build_ref.sh into oracle/_ref/).
//
// The reference file is included unmodified with its main() renamed, and
// compiled against the host-only SYCL stand-in in oracle/sycl_shim.  For a
// size n the driver writes, as raw float32 row-major files:
//   <out>_host.f32    the reference's host verification loop result
//                     (gemm(), mm2_cpu(), mm3_cpu(), syrk(), syr2k(),
//                     covariance(), correlation(); matmulchain: the identity
//                     its verify() expects)
//   <out>_device.f32  the output buffer after the reference's run() kernels
//                     executed on the host (its --device=cpu semantics)
// Covariance and correlation write their (n + 1) x (n + 1) symmat arrays;
// the matrix-vector benchmarks their output vectors (bicg: s then q; mvt: x1
// then x2).  The device output is read from the buffers setup() created, by
// creation index.
// and prints "verify=PASS|FAIL" from the reference's own verify().
// With --main it instead runs the reference's main() with the remaining
// arguments (its CLI, result consumers and timing harness).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <sycl/sycl.hpp>

#if defined(REF_MATMULCHAIN)
// runtime/matmulchain.cpp's main() ends without a return statement, which
// only main may do; renamed, it would run off the end of an int function.
// Its body is compiled as a void lambda instead.
#define main(...) reference_main_unused = 0; static auto reference_main_body = [](__VA_ARGS__) -> void
#include REF_SOURCE
;
#undef main
static int reference_main(int argc, char** argv) {
  reference_main_body(argc, argv);
  return 0;
}
#else
#define main reference_main
#include REF_SOURCE
#undef main
#endif

namespace {

void write_f32(const std::string& path, const float* p, size_t n) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if(!f) {
    std::perror(path.c_str());
    std::exit(2);
  }
  std::fwrite(p, sizeof(float), n, f);
  std::fclose(f);
}

BenchmarkArgs make_args(size_t n) {
  std::string size = "--size=" + std::to_string(n);
  const char* argv[] = {"ref", size.c_str(), "--device=cpu", "--num-runs=1"};
  return BenchmarkCommandLine{4, const_cast<char**>(argv)}.getBenchmarkArgs();
}

// run(events) where the benchmark records per-command events, run() otherwise
// (include/benchmark_traits.h:9-18).
template <class B>
auto run_commands(B& b) -> decltype(b.run(std::declval<std::vector<sycl::event>&>()), void()) {
  std::vector<sycl::event> events;
  b.run(events);
}
template <class B>
auto run_commands(B& b) -> decltype(b.run(), void()) {
  b.run();
}

}  // namespace

int main(int argc, char** argv) {
  if(argc >= 2 && std::strcmp(argv[1], "--main") == 0) {
    argv[1] = argv[0];
    return reference_main(argc - 1, argv + 1);
  }
  if(argc < 3) {
    std::fprintf(stderr, "usage: %s <n> <out-prefix> | --main <reference args...>\n", argv[0]);
    return 2;
  }
  const size_t n = std::strtoull(argv[1], nullptr, 10);
  const std::string out = argv[2];
  size_t nn = n * n;

  // 1) host verification loop, on freshly initialised inputs
  std::vector<float> host_out(nn);
#if defined(REF_GEMM)
  {
    std::vector<float> A(nn), B(nn), C(nn);
    init(A.data(), B.data(), C.data(), n);
    gemm(A.data(), B.data(), C.data(), n);
    host_out = C;
  }
  using Bench = Polybench_Gemm;
  const std::vector<size_t> out_index = {2};
#elif defined(REF_2MM)
  {
    std::vector<float> A(nn), B(nn), C(nn), D(nn), E(nn);
    init_array(A.data(), B.data(), C.data(), D.data(), n);
    mm2_cpu(A.data(), B.data(), C.data(), D.data(), E.data(), n);
    host_out = E;
  }
  using Bench = Polybench_2mm;
  const std::vector<size_t> out_index = {4};
#elif defined(REF_3MM)
  {
    std::vector<float> A(nn), B(nn), C(nn), D(nn), E(nn), F(nn), G(nn);
    init_array(A.data(), B.data(), C.data(), D.data(), n);
    mm3_cpu(A.data(), B.data(), C.data(), D.data(), E.data(), F.data(), G.data(), n);
    host_out = G;
  }
  using Bench = Polybench_3mm;
  const std::vector<size_t> out_index = {6};
#elif defined(REF_SYRK)
  {
    std::vector<float> A(nn), C(nn);
    init_arrays(A.data(), C.data(), n);
    syrk(A.data(), C.data(), n);
    host_out = C;
  }
  using Bench = Polybench_Syrk;
  const std::vector<size_t> out_index = {1};
#elif defined(REF_SYR2K)
  {
    std::vector<float> A(nn), B(nn), C(nn);
    init_arrays(A.data(), B.data(), C.data(), n);
    syr2k(A.data(), B.data(), C.data(), n);
    host_out = C;
  }
  using Bench = Polybench_Syr2k;
  const std::vector<size_t> out_index = {2};
#elif defined(REF_COVARIANCE)
  nn = (n + 1) * (n + 1);
  {
    std::vector<float> data(nn), symmat(nn), mean(n + 1);
    init_arrays(data.data(), n);
    covariance(data.data(), symmat.data(), mean.data(), n);
    host_out = symmat;
  }
  using Bench = Polybench_Covariance;
  const std::vector<size_t> out_index = {1};
#elif defined(REF_CORRELATION)
  nn = (n + 1) * (n + 1);
  {
    std::vector<float> data(nn), mean(n + 1), stddev(n + 1), symmat(nn);
    init_arrays(data.data(), n);
    correlation(data.data(), mean.data(), stddev.data(), symmat.data(), n);
    host_out = symmat;
  }
  using Bench = Polybench_Correlation;
  const std::vector<size_t> out_index = {3};
#elif defined(REF_MATMULCHAIN)
  for(size_t i = 0; i < n; ++i) host_out[i * n + i] = 1.f;
  using Bench = MatmulChain<float>;
  const std::vector<size_t> out_index = {4};
#elif defined(REF_ATAX)
  {
    std::vector<float> A(nn), x(n), y(n), tmp(n);
    init_array(x.data(), A.data(), n);
    atax_cpu(A.data(), x.data(), y.data(), tmp.data(), n);
    host_out = y;
  }
  using Bench = Polybench_Atax;
  const std::vector<size_t> out_index = {2};
#elif defined(REF_BICG)
  {
    std::vector<float> A(nn), p(n), r(n), s(n), q(n);
    init_array(A.data(), p.data(), r.data(), n);
    bicg_cpu(A.data(), r.data(), s.data(), p.data(), q.data(), n);
    host_out = s;
    host_out.insert(host_out.end(), q.begin(), q.end());
  }
  using Bench = Polybench_Bicg;
  const std::vector<size_t> out_index = {2, 4};
#elif defined(REF_MVT)
  {
    std::vector<float> a(nn), x1(n), x2(n), y1(n), y2(n);
    init_arrays(a.data(), x1.data(), x2.data(), y1.data(), y2.data(), n);
    runMvt(a.data(), x1.data(), x2.data(), y1.data(), y2.data(), n);
    host_out = x1;
    host_out.insert(host_out.end(), x2.begin(), x2.end());
  }
  using Bench = Polybench_Mvt;
  const std::vector<size_t> out_index = {1, 2};
#elif defined(REF_GESUMMV)
  {
    std::vector<float> A(nn), B(nn), x(n), y(n), tmp(n);
    init(A.data(), B.data(), x.data(), n);
    gesummv(A.data(), B.data(), x.data(), y.data(), tmp.data(), n);
    host_out = y;
  }
  using Bench = Polybench_Gesummv;
  const std::vector<size_t> out_index = {3};
#else
#error "define the REF_<benchmark> macro of the included source"
#endif
  write_f32(out + "_host.f32", host_out.data(), host_out.size());

  // 2) the benchmark's own setup / run / verify with the kernels on the host
  BenchmarkArgs args = make_args(n);
  Bench b(args);
  const size_t first = sycl::detail::buffer_log().size();
  b.setup();
  const auto t0 = std::chrono::steady_clock::now();
  run_commands(b);
  args.device_queue.wait_and_throw();
  const auto t1 = std::chrono::steady_clock::now();
  std::vector<float> dev_out;
  for(size_t idx : out_index) {
    const auto& st = *sycl::detail::buffer_log().at(first + idx);
    const float* p = static_cast<const float*>(st.data);
    dev_out.insert(dev_out.end(), p, p + st.count);
  }
  write_f32(out + "_device.f32", dev_out.data(), dev_out.size());
  VerificationSetting vs{true, {0, 0, 0}, {1, 1, 1}};
  const bool ok = b.verify(vs);
  std::printf("verify=%s kernel_seconds=%.6f\n", ok ? "PASS" : "FAIL",
      std::chrono::duration<double>(t1 - t0).count());
  return 0;
}
