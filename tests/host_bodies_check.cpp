// The --device=cpu kernel bodies of polybench_common.h against the
// per-element loops of the reference kernels they restate, bit for bit:
//   host_gemm_body(tb = true)  syrk.cpp:74-83    C = beta C + sum_k (alpha A[i][k]) A[j][k]
//   host_syr2k_body            syr2k.cpp:78-87   one statement per k
//   host_gemv_t_body           atax.cpp:87-95, bicg.cpp:77-84
//   host_gemv_n_body           atax.cpp:73-84, bicg.cpp:89-97, mvt.cpp:75-96
//   host_gesummv_body          gesummv.cpp:84-98
//   host_xtx_upper             covariance.cpp:114-126 (skip 0), correlation.cpp:167-181 (skip 1)
//   host_column_sums           the column means and standard deviations, covariance.cpp:80-96 and
//                              correlation.cpp:107-142
// Built with the executables' flags (-O3 -fopenmp -ffp-contract=off); exit
// status = number of mismatching cases.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "polybench_common.h"

namespace {

template <class T>
void loop_syrk(std::size_t n, T alpha, const T* A, T beta, T* C) {
  for(std::size_t i = 0; i < n; ++i)
    for(std::size_t j = 0; j < n; ++j) {
      T acc = C[i * n + j] * beta;
      for(std::size_t k = 0; k < n; ++k) acc += (alpha * A[i * n + k]) * A[j * n + k];
      C[i * n + j] = acc;
    }
}

template <class T>
void loop_syr2k(std::size_t n, T alpha, const T* A, const T* B, T beta, T* C) {
  for(std::size_t i = 0; i < n; i++)
    for(std::size_t j = 0; j < n; j++) {
      T c = C[i * n + j] * beta;
      for(std::size_t k = 0; k < n; k++) c += alpha * A[i * n + k] * B[j * n + k] + alpha * B[i * n + k] * A[j * n + k];
      C[i * n + j] = c;
    }
}

void loop_gemv_t(std::size_t n, const float* A, const float* x, float* y) {
  for(std::size_t j = 0; j < n; ++j)
    for(std::size_t i = 0; i < n; i++) y[j] += A[i * n + j] * x[i];
}

void loop_gemv_n(std::size_t n, const float* A, const float* x, float* y) {
  for(std::size_t i = 0; i < n; ++i)
    for(std::size_t j = 0; j < n; j++) y[i] += A[i * n + j] * x[j];
}

void loop_gesummv(std::size_t n, float alpha, float beta, const float* A, const float* B, const float* x, float* tmp,
    float* y) {
  for(std::size_t i = 0; i < n; ++i) {
    for(std::size_t j = 0; j < n; j++) {
      tmp[i] += A[i * n + j] * x[j];
      y[i] += B[i * n + j] * x[j];
    }
    y[i] = alpha * tmp[i] + beta * y[i];
  }
}

void loop_xtx(std::size_t n, std::size_t ld, const float* X, float* S, std::size_t skip) {
  for(std::size_t j1 = 0; j1 < n; ++j1)
    for(std::size_t j2 = j1 + skip; j2 < n; j2++) {
      S[j1 * ld + j2] = 0.0f;
      for(std::size_t i = 0; i < n; i++) S[j1 * ld + j2] += X[i * ld + j1] * X[i * ld + j2];
      S[j2 * ld + j1] = S[j1 * ld + j2];
    }
}

void loop_column_sums(std::size_t n, std::size_t ld, const float* X, float* col, const float* mu) {
  for(std::size_t j = 0; j < n; ++j)
    for(std::size_t i = 0; i < n; i++)
      col[j] += mu ? (X[i * ld + j] - mu[j]) * (X[i * ld + j] - mu[j]) : X[i * ld + j];
}

template <class T>
std::vector<T> normal(std::size_t count, unsigned seed) {
  std::mt19937 g(seed);
  std::normal_distribution<double> d;
  std::vector<T> v(count);
  for(auto& x : v) x = T(d(g));
  return v;
}

int report(const char* what, std::size_t n, const void* a, const void* b, std::size_t bytes) {
  const bool same = std::memcmp(a, b, bytes) == 0;
  std::printf("%-12s n=%-4zu %s\n", what, n, same ? "bitwise equal" : "MISMATCH");
  return same ? 0 : 1;
}

template <class T>
int check_symmetric(std::size_t n) {
  const auto A = normal<T>(n * n, unsigned(n)), B = normal<T>(n * n, unsigned(n) + 1),
             C = normal<T>(n * n, unsigned(n) + 2);
  const T alpha = T(1.5), beta = T(-0.75);
  int bad = 0;
  auto c1 = C, c2 = C;
  loop_syrk(n, alpha, A.data(), beta, c1.data());
  poly::host_gemm_body<T>(n, true, alpha, A.data(), A.data(), beta, c2.data());
  bad += report(sizeof(T) == 4 ? "syrk f32" : "syrk f64", n, c1.data(), c2.data(), c1.size() * sizeof(T));
  c1 = C, c2 = C;
  loop_syr2k(n, alpha, A.data(), B.data(), beta, c1.data());
  poly::host_syr2k_body<T>(n, alpha, A.data(), B.data(), beta, c2.data());
  bad += report(sizeof(T) == 4 ? "syr2k f32" : "syr2k f64", n, c1.data(), c2.data(), c1.size() * sizeof(T));
  return bad;
}

int check_columns(std::size_t n) {
  const auto A = normal<float>(n * n, unsigned(n) + 3), x = normal<float>(n, unsigned(n) + 4),
             y = normal<float>(n, unsigned(n) + 5);
  auto y1 = y, y2 = y;
  loop_gemv_t(n, A.data(), x.data(), y1.data());
  poly::host_gemv_t_body(n, A.data(), x.data(), y2.data());
  int bad = report("gemv_t", n, y1.data(), y2.data(), n * 4);
  y1 = y, y2 = y;
  loop_gemv_n(n, A.data(), x.data(), y1.data());
  poly::host_gemv_n_body(n, A.data(), x.data(), y2.data());
  bad += report("gemv_n", n, y1.data(), y2.data(), n * 4);
  const auto B = normal<float>(n * n, unsigned(n) + 8), tmp = normal<float>(n, unsigned(n) + 9);
  auto t1 = tmp, t2 = tmp;
  y1 = y, y2 = y;
  loop_gesummv(n, 1.25f, -0.5f, A.data(), B.data(), x.data(), t1.data(), y1.data());
  poly::host_gesummv_body(n, 1.25f, -0.5f, A.data(), B.data(), x.data(), t2.data(), y2.data());
  bad += report("gesummv", n, y1.data(), y2.data(), n * 4) + report("gesummv tmp", n, t1.data(), t2.data(), n * 4);
  // X^T X on the interior of an (n+1) x (n+1) array, as covariance/correlation
  const std::size_t ld = n + 1;
  const auto X = normal<float>(ld * ld, unsigned(n) + 6);
  for(std::size_t skip : {0, 1}) {
    std::vector<float> s1(ld * ld, 7.f), s2(ld * ld, 7.f);
    loop_xtx(n, ld, X.data() + ld + 1, s1.data() + ld + 1, skip);
    poly::host_xtx_upper(n, ld, X.data() + ld + 1, s2.data() + ld + 1, skip);
    bad += report(skip ? "xtx skip 1" : "xtx skip 0", n, s1.data(), s2.data(), s1.size() * 4);
  }
  // column sums (means) and squared deviations (standard deviations)
  const auto mu = normal<float>(n, unsigned(n) + 7);
  std::vector<float> m1(n, 0.25f), m2(n, 0.25f);
  loop_column_sums(n, ld, X.data() + ld + 1, m1.data(), nullptr);
  poly::host_column_sums(n, n, ld, X.data() + ld + 1, m2.data(), [](float v, std::size_t) { return v; });
  bad += report("column sum", n, m1.data(), m2.data(), n * 4);
  std::vector<float> d1(n, 0.f), d2(n, 0.f);
  loop_column_sums(n, ld, X.data() + ld + 1, d1.data(), mu.data());
  const float* m = mu.data();
  poly::host_column_sums(n, n, ld, X.data() + ld + 1, d2.data(),
      [m](float v, std::size_t j) { return (v - m[j]) * (v - m[j]); });
  bad += report("column dev", n, d1.data(), d2.data(), n * 4);
  return bad;
}

}  // namespace

int main() {
  int bad = 0;
  for(std::size_t n : {1, 2, 63, 64, 65, 130, 257}) {
    bad += check_symmetric<float>(n);
    bad += check_symmetric<double>(n);
    bad += check_columns(n);
  }
  return bad;
}
