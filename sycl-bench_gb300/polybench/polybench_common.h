// Shared pieces of the five PolyBench contraction benchmarks.
//
//  * percentDiff / absVal: the verification comparator of
//    polybench/common/polybenchUtilFuncts.h:27-42 (float narrowing kept).
//  * Benchmark-specific options, read through args.cli like the reference's
//    own extra options (include/command_line.h:98-103):
//      --precision=fp32|bf16x3|tf32|tf32x3|bf16x6|fp16x3|fp8[,...]  form(s) to run (fp32)
//      --init=polybench|uniform|normal          input initialisation (polybench)
//      --seed=<u64>                             seed of uniform/normal inputs (1)
//      --alpha=<f> --beta=<f>                   override syrk/syr2k/gemm scalars
//      --verification-oracle=host|fp64          host FP32 loop of the reference
//                                               (default) or an FP64 reference
//      --error-report=<file.jsonl>              append max/Frobenius error vs FP64
//      --graph                                  (2mm, 3mm, matmulchain) stages as one captured CUDA graph
//      --grouped                                (3mm, matmulchain) the independent stages as one grouped launch
//  * Memoised oracles: the reference recomputes its O(N^3) host loop after
//    every run (include/common.h:113-121); the result depends only on the
//    benchmark, size and inputs, so it is computed once per process.
//  * Host-device kernels for --device=cpu: the reference kernel bodies run
//    on the host cores (OpenMP over output rows, each element keeps its
//    sequential k order).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

#include "common.h"
#include "gbpoly.h"

// ------------------------------------------------------------- comparator --
#define SMALL_FLOAT_VAL 0.00000001f

inline float absVal(float a) { return a < 0 ? a * -1 : a; }

inline float percentDiff(double val1, double val2) {
  if(absVal(val1) < 0.01 && absVal(val2) < 0.01) return 0.0f;
  return 100.0f * absVal(absVal(val1 - val2) / absVal(val1 + SMALL_FLOAT_VAL));
}

namespace poly {

constexpr double kErrorThreshold = 0.05;  // percent (gemm.cpp:96 and the other four)

// ---------------------------------------------------------------- options --
enum class Init { Polybench, Uniform, Normal };

struct Options {
  gbpoly_precision precision = GBPOLY_PREC_FP32;
  Init init = Init::Polybench;
  uint64_t seed = 1;
  bool fp64_oracle = false;
  std::string error_report;
  bool has_alpha = false, has_beta = false;
  double alpha = 0, beta = 0;
};

inline const char* precision_name(gbpoly_precision p) {
  switch(p) {
  case GBPOLY_PREC_FP32: return "fp32";
  case GBPOLY_PREC_BF16X3: return "bf16x3";
  case GBPOLY_PREC_TF32: return "tf32";
  case GBPOLY_PREC_FP8: return "fp8";
  case GBPOLY_PREC_TF32X3: return "tf32x3";
  case GBPOLY_PREC_BF16X6: return "bf16x6";
  case GBPOLY_PREC_FP16X3: return "fp16x3";
  }
  return "?";
}

inline gbpoly_precision parse_precision(const std::string& s) {
  if(s == "fp32") return GBPOLY_PREC_FP32;
  if(s == "bf16x3") return GBPOLY_PREC_BF16X3;
  if(s == "tf32") return GBPOLY_PREC_TF32;
  if(s == "fp8") return GBPOLY_PREC_FP8;
  if(s == "tf32x3") return GBPOLY_PREC_TF32X3;
  if(s == "bf16x6") return GBPOLY_PREC_BF16X6;
  if(s == "fp16x3") return GBPOLY_PREC_FP16X3;
  throw std::invalid_argument{"unknown --precision value: " + s};
}

inline std::vector<gbpoly_precision> precisions(const BenchmarkArgs& args) {
  std::vector<gbpoly_precision> out;
  std::stringstream in(args.cli.getOrDefault<std::string>("--precision", "fp32"));
  std::string item;
  while(std::getline(in, item, ',')) out.push_back(parse_precision(item));
  return out;
}

// The matrix-vector benchmarks run the plain FP32 form only (HBM-bound, no
// contraction for the tensor cores): --precision may name fp32 alone.
// Precision forms whose split pass can centre (and scale) the columns of the
// covariance / correlation data itself (gbpoly_covariance_f32).
inline bool centres_in_split(gbpoly_precision p) {
  return p == GBPOLY_PREC_TF32 || p == GBPOLY_PREC_BF16X3 || p == GBPOLY_PREC_TF32X3 || p == GBPOLY_PREC_BF16X6 ||
         p == GBPOLY_PREC_FP16X3;
}

inline void require_fp32_only(const BenchmarkArgs& args) {
  for(auto p : precisions(args))
    if(p != GBPOLY_PREC_FP32)
      throw std::invalid_argument{"--precision: this benchmark has the fp32 form only"};
}

inline Options options(const BenchmarkArgs& args, gbpoly_precision prec) {
  Options o;
  o.precision = prec;
  const std::string init = args.cli.getOrDefault<std::string>("--init", "polybench");
  if(init == "polybench")
    o.init = Init::Polybench;
  else if(init == "uniform")
    o.init = Init::Uniform;
  else if(init == "normal")
    o.init = Init::Normal;
  else
    throw std::invalid_argument{"unknown --init value: " + init};
  o.seed = args.cli.getOrDefault<uint64_t>("--seed", 1);
  const std::string orc = args.cli.getOrDefault<std::string>("--verification-oracle", "host");
  if(orc != "host" && orc != "fp64") throw std::invalid_argument{"unknown --verification-oracle value: " + orc};
  o.fp64_oracle = orc == "fp64";
  o.error_report = args.cli.getOrDefault<std::string>("--error-report", "");
  o.has_alpha = args.cli.isArgSet("--alpha");
  o.has_beta = args.cli.isArgSet("--beta");
  if(o.has_alpha) o.alpha = args.cli.get<double>("--alpha");
  if(o.has_beta) o.beta = args.cli.get<double>("--beta");
  return o;
}

// Benchmark name: the reference's name for the default configuration, with
// suffixes for every non-default choice (element type, form, inputs, scalars).
template <class T>
std::string variant_name(const std::string& base, const Options& o) {
  std::string n = base;
  if(std::is_same<T, double>::value) n += std::string("_") + ReadableTypename<double>::name;
  if(o.precision != GBPOLY_PREC_FP32) n += std::string("_") + precision_name(o.precision);
  if(o.init == Init::Uniform) n += "_uniform_seed" + std::to_string(o.seed);
  if(o.init == Init::Normal) n += "_normal_seed" + std::to_string(o.seed);
  if(o.has_alpha || o.has_beta) {
    std::ostringstream s;
    s << "_ab" << (o.has_alpha ? o.alpha : 0) << "_" << (o.has_beta ? o.beta : 0);
    n += s.str();
  }
  return n;
}

// ------------------------------------------------------- seeded variants --
// splitmix64: a fixed, platform-independent stream.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform01() { return double(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
};

// Fill `count` values uniform in [-1, 1) or standard normal (Box-Muller),
// stream `which` of the seed (one stream per matrix).
template <class T>
void fill_random(T* p, std::size_t count, Init kind, uint64_t seed, uint64_t which) {
  Rng r(seed * 0x100000001B3ull + which * 0xC2B2AE3D27D4EB4Full + 7);
  if(kind == Init::Uniform) {
    for(std::size_t i = 0; i < count; ++i) p[i] = static_cast<T>(2.0 * r.uniform01() - 1.0);
  } else {
    for(std::size_t i = 0; i < count; i += 2) {
      const double u1 = 1.0 - r.uniform01(), u2 = r.uniform01();
      const double rad = std::sqrt(-2.0 * std::log(u1)), th = 6.283185307179586 * u2;
      p[i] = static_cast<T>(rad * std::cos(th));
      if(i + 1 < count) p[i + 1] = static_cast<T>(rad * std::sin(th));
    }
  }
}

// ------------------------------------------------------------ memoisation --
template <class T>
std::shared_ptr<const std::vector<T>> memo(const std::string& key, const std::function<std::vector<T>()>& make) {
  static std::map<std::string, std::shared_ptr<const std::vector<T>>> cache;
  auto it = cache.find(key);
  if(it != cache.end()) return it->second;
  auto v = std::make_shared<const std::vector<T>>(make());
  cache[key] = v;
  return v;
}

inline std::string memo_key(const std::string& name, std::size_t n, const Options& o, const char* kind) {
  return name + "|" + std::to_string(n) + "|" + std::to_string(int(o.init)) + "|" + std::to_string(o.seed) + "|" +
         std::to_string(o.alpha) + "|" + std::to_string(o.beta) + "|" + kind;
}

// ----------------------------------------------------------- verification --
// Row-major walk, first element over the threshold fails (gemm.cpp:107-113).
template <class T, class R>
bool compare(const R* reference, const T* device, std::size_t count) {
  for(std::size_t i = 0; i < count; ++i)
    if(percentDiff(reference[i], device[i]) > kErrorThreshold) return false;
  return true;
}

struct ErrorNorms {
  double max_rel = 0, frob_rel = 0, max_elem_rel = 0;
};

template <class T>
ErrorNorms error_norms(const T* c, const double* r, std::size_t count) {
  double me = 0, mr = 0, se = 0, sr = 0, mer = 0;
  bool bad = false;
  for(std::size_t i = 0; i < count; ++i) {
    const double e = std::fabs(double(c[i]) - r[i]), a = std::fabs(r[i]);
    if(!std::isfinite(e)) bad = true;
    me = std::max(me, e);
    mr = std::max(mr, a);
    se += e * e;
    sr += a * a;
    if(a > 0) mer = std::max(mer, e / a);
  }
  ErrorNorms n;
  if(bad) {
    n.max_rel = n.frob_rel = n.max_elem_rel = HUGE_VAL;
    return n;
  }
  n.max_rel = mr > 0 ? me / mr : me;
  n.frob_rel = sr > 0 ? std::sqrt(se / sr) : std::sqrt(se);
  n.max_elem_rel = mer;
  return n;
}

// One line per benchmark configuration and process: verify() runs after
// every run (as the reference harness does, common.h:116), and the later
// runs recompute the same norms.  The double variants (names carrying the
// "_fp64" suffix variant_name gives them) are labelled "fp64".
inline void append_error_report(const Options& o, const std::string& bench, std::size_t n, const std::string& device,
    const ErrorNorms& e, bool passed) {
  if(o.error_report.empty()) return;
  static std::set<std::string> written;
  if(!written.insert(o.error_report + "|" + bench + "|" + std::to_string(n)).second) return;
  const bool fp64 = bench.find(std::string("_") + ReadableTypename<double>::name) != std::string::npos;
  std::ofstream f(o.error_report, std::ios::app);
  char buf[768];
  snprintf(buf, sizeof buf,
      "{\"benchmark\": \"%s\", \"size\": %zu, \"precision\": \"%s\", \"init\": \"%s\", \"seed\": %llu, "
      "\"device\": \"%s\", \"max_rel\": %.6e, \"frob_rel\": %.6e, \"max_elem_rel\": %.6e, \"verification\": \"%s\"}",
      bench.c_str(), n, fp64 ? ReadableTypename<double>::name : precision_name(o.precision),
      o.init == Init::Polybench ? "polybench" : (o.init == Init::Uniform ? "uniform" : "normal"),
      (unsigned long long)o.seed, device.c_str(), e.max_rel, e.frob_rel, e.max_elem_rel, passed ? "PASS" : "FAIL");
  f << buf << "\n";
}

// ---------------------------------------------------- FP64 reference steps --
// A device-side FP64 contraction sequence over N x N matrices, used for the
// FP64 oracle on the GPU: upload FP32 inputs as FP64, run DGEMMs, read back.
class Fp64Device {
public:
  Fp64Device(const gb::Queue& q, std::size_t n) : q_(q), n_(n) {}
  ~Fp64Device() {
    for(void* p : owned_) gbpoly_free(q_.ctx(), p);
  }
  template <class T>
  double* upload(const T* host) {
    double* d = alloc();
    if(std::is_same<T, double>::value) {
      gb::check(gbpoly_memcpy_h2d(q_.ctx(), d, host, bytes()), "h2d");
    } else {
      float* tmp = nullptr;
      gb::check(gbpoly_malloc(q_.ctx(), reinterpret_cast<void**>(&tmp), n_ * n_ * sizeof(float)), "malloc");
      owned_.push_back(tmp);
      gb::check(gbpoly_memcpy_h2d(q_.ctx(), tmp, host, n_ * n_ * sizeof(float)), "h2d");
      gb::check(gbpoly_convert_f32_f64(q_.ctx(), tmp, d, int64_t(n_ * n_)), "convert");
    }
    return d;
  }
  double* zeros() {
    double* d = alloc();
    gb::check(gbpoly_memset(q_.ctx(), d, 0, bytes()), "memset");
    return d;
  }
  // C = alpha * op(A) op(B) + beta * C
  void gemm(gbpoly_op oa, gbpoly_op ob, double alpha, const double* A, const double* B, double beta, double* C) {
    const int64_t n = int64_t(n_);
    gb::check(gbpoly_gemm_f64(q_.ctx(), oa, ob, n, n, n, alpha, A, n, B, n, beta, C, n), "dgemm");
  }
  std::vector<double> download(const double* d) {
    std::vector<double> h(n_ * n_);
    gb::check(gbpoly_memcpy_d2h(q_.ctx(), h.data(), d, bytes()), "d2h");
    q_.wait_and_throw();
    return h;
  }

private:
  std::size_t bytes() const { return n_ * n_ * sizeof(double); }
  double* alloc() {
    double* d = nullptr;
    gb::check(gbpoly_malloc(q_.ctx(), reinterpret_cast<void**>(&d), bytes()), "malloc");
    owned_.push_back(d);
    return d;
  }
  gb::Queue q_;
  std::size_t n_;
  std::vector<void*> owned_;
};

// Host FP64 contraction C = alpha * op(A) op(B) + beta * C (N x N), OpenMP over rows.
template <class TA>
void host_gemm_f64(std::size_t n, bool ta, bool tb, double alpha, const TA* A, const TA* B, double beta,
    std::vector<double>& C) {
#pragma omp parallel for schedule(static)
  for(long i = 0; i < long(n); ++i)
    for(std::size_t j = 0; j < n; ++j) {
      double s = 0;
      for(std::size_t k = 0; k < n; ++k)
        s += double(ta ? A[k * n + i] : A[i * n + k]) * double(tb ? B[j * n + k] : B[k * n + j]);
      C[i * n + j] = alpha * s + beta * C[i * n + j];
    }
}

// ------------------------------------------------- host-device kernel bodies --
// Bt = B^T for n x n row-major B, in 32 x 32 blocks, OpenMP over block rows.
template <class T>
std::vector<T> host_transpose(std::size_t n, const T* B) {
  std::vector<T> t(n * n);
  constexpr std::size_t W = 32;
#pragma omp parallel for schedule(static)
  for(long r0 = 0; r0 < long(n); r0 += long(W))
    for(std::size_t c0 = 0; c0 < n; c0 += W)
      for(std::size_t r = std::size_t(r0); r < std::min(n, std::size_t(r0) + W); ++r)
        for(std::size_t c = c0; c < std::min(n, c0 + W); ++c) t[c * n + r] = B[r * n + c];
  return t;
}

// C[i][j] = beta*C[i][j] + sum_k (alpha*op(A)[i][k]) * op(B)[k][j], each element
// walking k in order; OpenMP over rows, 64-wide column blocks vectorised.  A
// transposed B (syrk's A A^T) is transposed once first, so the column block
// reads contiguous rows: the same operations on every element.
template <class T>
void host_gemm_body(std::size_t n, bool tb, T alpha, const T* A, const T* B, T beta, T* C) {
  std::vector<T> bt;
  if(tb) {
    bt = host_transpose(n, B);
    B = bt.data();
  }
  constexpr std::size_t V = 64;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < long(n); ++i) {
    for(std::size_t j0 = 0; j0 < n; j0 += V) {
      const std::size_t j1 = std::min(n, j0 + V);
      T acc[V];
      for(std::size_t j = j0; j < j1; ++j) acc[j - j0] = C[i * n + j] * beta;
      for(std::size_t k = 0; k < n; ++k) {
        const T a = alpha * A[i * n + k];
        const T* b = B + k * n;
        for(std::size_t j = j0; j < j1; ++j) acc[j - j0] += a * b[j];
      }
      for(std::size_t j = j0; j < j1; ++j) C[i * n + j] = acc[j - j0];
    }
  }
}

// C[i][j] = beta*C[i][j] + sum_k (alpha*A[i][k]*B[j][k] + alpha*B[i][k]*A[j][k])
// with k in order and one statement per k (syr2k.cpp:78-87).  A and B are
// transposed once so that a 64-wide block of j reads contiguous rows of Aᵀ
// and Bᵀ; the operations per element are those of the per-element loop.
template <class T>
void host_syr2k_body(std::size_t n, T alpha, const T* A, const T* B, T beta, T* C) {
  const std::vector<T> at = host_transpose(n, A), bt = host_transpose(n, B);
  constexpr std::size_t V = 64;
#pragma omp parallel for schedule(static)
  for(long i = 0; i < long(n); i++)
    for(std::size_t j0 = 0; j0 < n; j0 += V) {
      const std::size_t j1 = std::min(n, j0 + V);
      T c[V];
      for(std::size_t j = j0; j < j1; j++) c[j - j0] = C[i * n + j] * beta;
      for(std::size_t k = 0; k < n; k++) {
        const T a = alpha * A[i * n + k], b = alpha * B[i * n + k];
        const T *bk = bt.data() + k * n, *ak = at.data() + k * n;
        for(std::size_t j = j0; j < j1; j++) c[j - j0] += a * bk[j] + b * ak[j];
      }
      for(std::size_t j = j0; j < j1; j++) C[i * n + j] = c[j - j0];
    }
}

// y[j] += A[i][j] * x[i] for an n x n row-major A, i in order for each j: the
// transposed matrix-vector kernels (atax.cpp:87-95, bicg.cpp:77-84).  A thread
// owns a block of 64 columns and walks the rows, so each row segment is one
// contiguous read instead of one cache line per element.
inline void host_gemv_t_body(std::size_t n, const float* A, const float* x, float* y) {
  constexpr std::size_t V = 64;
  const long blocks = long((n + V - 1) / V);
#pragma omp parallel for schedule(static)
  for(long b = 0; b < blocks; ++b) {
    const std::size_t j0 = std::size_t(b) * V, j1 = std::min(n, j0 + V);
    float acc[V];
    for(std::size_t j = j0; j < j1; j++) acc[j - j0] = y[j];
    for(std::size_t i = 0; i < n; i++) {
      const float xi = x[i];
      const float* row = A + i * n;
      for(std::size_t j = j0; j < j1; j++) acc[j - j0] += row[j] * xi;
    }
    for(std::size_t j = j0; j < j1; j++) y[j] = acc[j - j0];
  }
}

// y[i] += A[i][j] * x[j] for an n x n row-major A, j in order for each i:
// the row kernels of atax.cpp:73-84, bicg.cpp:89-97 and mvt.cpp:75-96.  Each
// row is a chain of dependent adds, so a thread carries 8 rows at once (8
// independent chains) instead of waiting on one; every row keeps its order.
inline void host_gemv_n_body(std::size_t n, const float* A, const float* x, float* y) {
  constexpr std::size_t R = 8;
  const long groups = long((n + R - 1) / R);
#pragma omp parallel for schedule(static)
  for(long g = 0; g < groups; ++g) {
    const std::size_t i0 = std::size_t(g) * R;
    if(i0 + R <= n) {
      float acc[R];
      for(std::size_t r = 0; r < R; ++r) acc[r] = y[i0 + r];
      for(std::size_t j = 0; j < n; ++j) {
        const float xj = x[j];
#pragma GCC unroll 8
        for(std::size_t r = 0; r < R; ++r) acc[r] += A[(i0 + r) * n + j] * xj;
      }
      for(std::size_t r = 0; r < R; ++r) y[i0 + r] = acc[r];
    } else {
      for(std::size_t i = i0; i < n; ++i)
        for(std::size_t j = 0; j < n; ++j) y[i] += A[i * n + j] * x[j];
    }
  }
}

// gesummv.cpp:84-98 on the host: tmp[i] += A[i][j] x[j] and y[i] += B[i][j] x[j]
// with j in order, then y[i] = alpha tmp[i] + beta y[i]; 4 rows per thread at
// once (8 independent chains), each row in its own order.
inline void host_gesummv_body(std::size_t n, float alpha, float beta, const float* A, const float* B, const float* x,
    float* tmp, float* y) {
  constexpr std::size_t R = 4;
  const long groups = long((n + R - 1) / R);
#pragma omp parallel for schedule(static)
  for(long g = 0; g < groups; ++g) {
    const std::size_t i0 = std::size_t(g) * R, i1 = std::min(n, i0 + R);
    if(i1 - i0 == R) {
      float t[R], u[R];
      for(std::size_t r = 0; r < R; ++r) t[r] = tmp[i0 + r], u[r] = y[i0 + r];
      for(std::size_t j = 0; j < n; ++j) {
        const float xj = x[j];
#pragma GCC unroll 4
        for(std::size_t r = 0; r < R; ++r) {
          t[r] += A[(i0 + r) * n + j] * xj;
          u[r] += B[(i0 + r) * n + j] * xj;
        }
      }
      for(std::size_t r = 0; r < R; ++r) tmp[i0 + r] = t[r], y[i0 + r] = u[r];
    } else {
      for(std::size_t i = i0; i < i1; ++i)
        for(std::size_t j = 0; j < n; ++j) {
          tmp[i] += A[i * n + j] * x[j];
          y[i] += B[i * n + j] * x[j];
        }
    }
    for(std::size_t i = i0; i < i1; ++i) y[i] = alpha * tmp[i] + beta * y[i];
  }
}

// col[j] += term(X[i][j], j) for i = 0..rows-1 in order, each column of an
// rows x cols X (leading dimension ld): the column means and standard
// deviations of covariance.cpp:80-96 and correlation.cpp:107-142.  A thread
// owns a block of 64 columns and walks the rows (contiguous row segments).
template <class Term>
void host_column_sums(std::size_t rows, std::size_t cols, std::size_t ld, const float* X, float* col, Term term) {
  constexpr std::size_t V = 64;
  const long blocks = long((cols + V - 1) / V);
#pragma omp parallel for schedule(static)
  for(long b = 0; b < blocks; ++b) {
    const std::size_t j0 = std::size_t(b) * V, j1 = std::min(cols, j0 + V);
    float acc[V];
    for(std::size_t j = j0; j < j1; j++) acc[j - j0] = col[j];
    for(std::size_t i = 0; i < rows; i++) {
      const float* row = X + i * ld;
      for(std::size_t j = j0; j < j1; j++) acc[j - j0] += term(row[j], j);
    }
    for(std::size_t j = j0; j < j1; j++) col[j] = acc[j - j0];
  }
}

// S[j1][j2] = S[j2][j1] = sum_i X[i][j1] * X[i][j2] over n x n X (leading
// dimension ld) for j2 >= j1 + skip, each sum from 0 with i in order: the
// XᵀX kernels of covariance.cpp:114-126 (skip 0) and correlation.cpp:167-181
// (skip 1; the unit diagonal is the caller's).  OpenMP over j1, a 64-wide
// block of j2 vectorised over contiguous row segments; the same operations
// on every element as the per-element loop.
template <class T>
void host_xtx_upper(std::size_t n, std::size_t ld, const T* X, T* S, std::size_t skip) {
  constexpr std::size_t V = 64;
#pragma omp parallel for schedule(dynamic, 4)
  for(long j1 = 0; j1 < long(n); ++j1) {
    for(std::size_t b0 = std::size_t(j1) + skip; b0 < n; b0 += V) {
      const std::size_t b1 = std::min(n, b0 + V);
      T acc[V];
      for(std::size_t j = b0; j < b1; ++j) acc[j - b0] = T(0);
      for(std::size_t i = 0; i < n; ++i) {
        const T x = X[i * ld + std::size_t(j1)];
        const T* row = X + i * ld;
        for(std::size_t j = b0; j < b1; ++j) acc[j - b0] += x * row[j];
      }
      for(std::size_t j = b0; j < b1; ++j) {
        S[std::size_t(j1) * ld + j] = acc[j - b0];
        S[j * ld + std::size_t(j1)] = acc[j - b0];
      }
    }
  }
}

}  // namespace poly
