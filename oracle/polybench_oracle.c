/*
 * polybench_oracle.c — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of sycl-bench's PolyBench dense-contraction benchmarks,
 * used as the correctness oracle by the tests, by __graft_entry__.smoke()
 * and by bench.py's CPU-baseline leg.  Nothing on the GPU product path links
 * or calls this file.
 *
 * Every function follows one place of the reference (paths relative to the
 * sycl-bench project root) and keeps its floating-point operation order:
 *   - initialisers           polybench/gemm.cpp:18-40, 2mm.cpp:16-45,
 *                            3mm.cpp:17-47, syrk.cpp:18-31, syr2k.cpp:18-32
 *   - host reference loops   gemm.cpp:42-56, 2mm.cpp:47-69, 3mm.cpp:49-86,
 *                            syrk.cpp:33-51, syr2k.cpp:34-52
 *   - device kernel bodies   gemm.cpp:82-91, syrk.cpp:74-83, syr2k.cpp:78-87
 *     (run on host cores: the reference's --device=cpu path)
 *   - comparator             polybench/common/polybenchUtilFuncts.h:27-42
 *   - covariance, correlation polybench/covariance.cpp:20-60,
 *                            polybench/correlation.cpp:23-87 (init and the
 *                            host loop; their run() kernels perform the same
 *                            per-element operations in the same order)
 *   - matmulchain product    runtime/matmulchain.cpp:11-30, with its int
 *                            accumulator
 *   - atax, bicg, mvt,       polybench/atax.cpp:20-46, bicg.cpp:20-48,
 *     gesummv                mvt.cpp:16-42, gesummv.cpp:30-56 (init and host
 *                            loop; their run() kernels perform the same
 *                            per-element operations in the same order)
 *
 * Parallelism: OpenMP over output rows.  Each output element keeps the
 * reference's sequential k order, so results do not depend on the thread
 * count.  Build with -ffp-contract=off (no fused multiply-add) so the float
 * operations are exactly the reference's mul-then-add on every host ISA.
 *
 * Pinned against the reference itself: oracle/build_ref.sh compiles the
 * unmodified reference sources with a host-only SYCL shim, and
 * tests/golden/make_golden.py stores their outputs; tests/test_oracle.py
 * checks this file against those fixtures bit for bit.
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long idx_t;

/* ------------------------------------------------------------ comparator -- */

/* polybenchUtilFuncts.h:27-33: absolute value of a float argument. */
static float abs_val(float a) { return a < 0 ? a * -1 : a; }

/* polybenchUtilFuncts.h:36-42.  Arguments are double, every absVal narrows to
 * float, SMALL_FLOAT_VAL is 1e-8f added in double. */
float orc_percent_diff(double v1, double v2) {
  if(abs_val((float)v1) < 0.01 && abs_val((float)v2) < 0.01) return 0.0f;
  return 100.0f * abs_val(abs_val((float)(v1 - v2)) / abs_val((float)(v1 + 0.00000001f)));
}

/* The verify loops (e.g. gemm.cpp:107-113): row-major walk, first element whose
 * percentDiff exceeds `threshold` fails.  Returns that index or -1.  Also
 * reports the largest percentDiff seen over the whole array in *max_diff and
 * the number of failing elements in *n_fail (both extensions, for reporting). */
idx_t orc_verify(const float* host, const float* dev, idx_t count, double threshold, float* max_diff, idx_t* n_fail) {
  idx_t first = -1, fails = 0;
  float worst = 0.0f;
  for(idx_t i = 0; i < count; ++i) {
    const float d = orc_percent_diff(host[i], dev[i]);
    if(d > worst || d != d) worst = d;
    if(d > threshold) {
      if(first < 0) first = i;
      ++fails;
    }
  }
  if(max_diff) *max_diff = worst;
  if(n_fail) *n_fail = fails;
  return first;
}

/* -------------------------------------------------------------- initialisers */

/* gemm.cpp:18-40 */
void orc_gemm_init(float* A, float* B, float* C, idx_t n) {
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) A[i * n + j] = ((float)i * (float)j) / (float)n;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) B[i * n + j] = ((float)i * (float)j + 1) / (float)n;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) C[i * n + j] = ((float)i * (float)j + 2) / (float)n;
}

/* 2mm.cpp:16-45 (A, B, C, D; E is not initialised by the reference) */
void orc_mm2_init(float* A, float* B, float* C, float* D, idx_t n) {
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) A[i * n + j] = ((float)i * (float)j) / (float)n;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) B[i * n + j] = ((float)i * (float)(j + 1)) / (float)n;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) C[i * n + j] = ((float)i * (float)(j + 3)) / (float)n;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) D[i * n + j] = ((float)i * (float)(j + 2)) / (float)n;
}

/* 3mm.cpp:17-47: same formulas as 2mm's four inputs. */
void orc_mm3_init(float* A, float* B, float* C, float* D, idx_t n) { orc_mm2_init(A, B, C, D, n); }

/* syrk.cpp:18-31 */
void orc_syrk_init(float* A, float* C, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    for(idx_t j = 0; j < n; j++) A[i * n + j] = ((float)i * (float)j) / (float)n;
    for(idx_t j = 0; j < n; j++) C[i * n + j] = ((float)i * (float)j + 2) / (float)n;
  }
}

/* syr2k.cpp:18-32 */
void orc_syr2k_init(float* A, float* B, float* C, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    for(idx_t j = 0; j < n; j++) C[i * n + j] = ((float)i * (float)j + 2) / (float)n;
    for(idx_t j = 0; j < n; j++) {
      A[i * n + j] = ((float)i * (float)j) / (float)n;
      B[i * n + j] = ((float)i * (float)j + 1) / (float)n;
    }
  }
}

/* ------------------------------------------------------- host FP32 oracles -- */

/* gemm.cpp:42-56, ALPHA=32412, BETA=2123 (int macros promoted to float). */
void orc_gemm_host(const float* A, const float* B, float* C, idx_t n) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      C[i * n + j] *= 2123;
      for(idx_t k = 0; k < n; ++k) C[i * n + j] += 32412 * A[i * n + k] * B[k * n + j];
    }
}

/* 2mm.cpp:47-69: C += A.B in place, then E = C.D. */
void orc_mm2_host(const float* A, const float* B, float* C, const float* D, float* E, idx_t n) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++)
      for(idx_t k = 0; k < n; ++k) C[i * n + j] += A[i * n + k] * B[k * n + j];
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      E[i * n + j] = 0;
      for(idx_t k = 0; k < n; ++k) E[i * n + j] += C[i * n + k] * D[k * n + j];
    }
}

/* 3mm.cpp:49-86: E = A.B, F = C.D, G = E.F. */
void orc_mm3_host(const float* A, const float* B, const float* C, const float* D, float* E, float* F, float* G,
    idx_t n) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      E[i * n + j] = 0;
      for(idx_t k = 0; k < n; ++k) E[i * n + j] += A[i * n + k] * B[k * n + j];
    }
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      F[i * n + j] = 0;
      for(idx_t k = 0; k < n; ++k) F[i * n + j] += C[i * n + k] * D[k * n + j];
    }
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      G[i * n + j] = 0;
      for(idx_t k = 0; k < n; ++k) G[i * n + j] += E[i * n + k] * F[k * n + j];
    }
}

/* syrk.cpp:33-51, alpha=123, beta=14512 (float constants). */
void orc_syrk_host(const float* A, float* C, idx_t n) {
  const float alpha = 123, beta = 14512;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) C[i * n + j] *= beta;
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++)
      for(idx_t k = 0; k < n; k++) C[i * n + j] += alpha * A[i * n + k] * A[j * n + k];
}

/* syr2k.cpp:34-52, ALPHA=BETA=1, two separate accumulations per k. */
void orc_syr2k_host(const float* A, const float* B, float* C, idx_t n) {
  const float alpha = 1, beta = 1;
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) C[i * n + j] *= beta;
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++)
      for(idx_t k = 0; k < n; k++) {
        C[i * n + j] += alpha * A[i * n + k] * B[j * n + k];
        C[i * n + j] += alpha * B[i * n + k] * A[j * n + k];
      }
}

/* ------------------------------------------- device kernel bodies on CPU -- */
/* The reference's --device=cpu path runs each parallel_for body once per
 * output element; a SYCL CPU runtime vectorises work-items along the
 * innermost range dimension (j).  These restatements keep that shape: each
 * element walks k in order (same result as one work-item), work-items are
 * processed in blocks of kVec along j, rows [row_begin, row_end) only, so a
 * bounded sample of the output can be timed. */
enum { kVec = 64 };

/* gemm.cpp:82-91: C[i][j] = BETA*C; C += ALPHA*A[i][k]*B[k][j].
 * `alpha`, `beta` generalise the constants for the variant workloads. */
void orc_gemm_body(const float* A, const float* B, float* C, idx_t n, idx_t row_begin, idx_t row_end, float alpha,
    float beta) {
  const idx_t nblk = (n + kVec - 1) / kVec;
#pragma omp parallel for collapse(2) schedule(static)
  for(idx_t i = row_begin; i < row_end; i++)
    for(idx_t jb = 0; jb < nblk; jb++) {
      const idx_t j0 = jb * kVec, j1 = (j0 + kVec < n) ? j0 + kVec : n;
      float acc[kVec];
      for(idx_t j = j0; j < j1; j++) acc[j - j0] = C[i * n + j] * beta;
      for(idx_t k = 0; k < n; k++) {
        const float a = alpha * A[i * n + k];
        const float* b = B + k * n;
        for(idx_t j = j0; j < j1; j++) acc[j - j0] += a * b[j];
      }
      for(idx_t j = j0; j < j1; j++) C[i * n + j] = acc[j - j0];
    }
}

/* syrk.cpp:74-83: C = beta*C; C += alpha*A[i][k]*A[j][k]. */
void orc_syrk_body(const float* A, float* C, idx_t n, idx_t row_begin, idx_t row_end, float alpha, float beta) {
#pragma omp parallel for collapse(2) schedule(static)
  for(idx_t i = row_begin; i < row_end; i++)
    for(idx_t j = 0; j < n; j++) {
      float c = C[i * n + j] * beta;
      for(idx_t k = 0; k < n; k++) c += alpha * A[i * n + k] * A[j * n + k];
      C[i * n + j] = c;
    }
}

/* syr2k.cpp:78-87: one statement per k, C += a*A_ik*B_jk + a*B_ik*A_jk. */
void orc_syr2k_body(const float* A, const float* B, float* C, idx_t n, idx_t row_begin, idx_t row_end, float alpha,
    float beta) {
#pragma omp parallel for collapse(2) schedule(static)
  for(idx_t i = row_begin; i < row_end; i++)
    for(idx_t j = 0; j < n; j++) {
      float c = C[i * n + j] * beta;
      for(idx_t k = 0; k < n; k++) c += alpha * A[i * n + k] * B[j * n + k] + alpha * B[i * n + k] * A[j * n + k];
      C[i * n + j] = c;
    }
}

/* ---------------------------------------------- covariance / correlation -- */
/* The data and symmat arrays are (n + 1) x (n + 1), used from index 1. */

static const float kCovFloatN = 3214212.01f;  /* covariance.cpp:18, a float constant */

/* covariance.cpp:20-29: rows and columns 0..n-1 written, the rest left as
 * the caller's zeros. */
void orc_covariance_init(float* data, idx_t n) {
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) data[i * (n + 1) + j] = ((float)i * (float)j) / (float)n;
}

/* covariance.cpp:31-60: column means over rows 1..n divided by float_n,
 * centring, then symmat[j1][j2] (j2 >= j1) as a sequential sum over rows,
 * mirrored.  `data` is centred in place. */
void orc_covariance_host(float* data, float* symmat, float* mean, idx_t n) {
  const idx_t ld = n + 1;
  for(idx_t j = 1; j <= n; j++) {
    mean[j] = 0.0f;
    for(idx_t i = 1; i <= n; i++) mean[j] += data[i * ld + j];
    mean[j] /= kCovFloatN;
  }
  for(idx_t i = 1; i <= n; i++)
    for(idx_t j = 1; j <= n; j++) data[i * ld + j] -= mean[j];
#pragma omp parallel for schedule(dynamic, 4)
  for(idx_t j1 = 1; j1 <= n; j1++)
    for(idx_t j2 = j1; j2 <= n; j2++) {
      float acc = 0.0f;
      for(idx_t i = 1; i <= n; i++) acc += data[i * ld + j1] * data[i * ld + j2];
      symmat[j1 * ld + j2] = acc;
      symmat[j2 * ld + j1] = acc;
    }
}

static const double kCorrFloatN = 3214212.01; /* correlation.cpp:12, a double constant */
static const double kCorrEps = 0.005;         /* correlation.cpp:13 */

/* correlation.cpp:23-33: written with a row stride of n (not n + 1) over
 * i, j in 0..n, so each row's last value lands on the next row's first
 * slot, which the next row then overwrites. */
void orc_correlation_init(float* data, idx_t n) {
  for(idx_t i = 0; i <= n; i++)
    for(idx_t j = 0; j <= n; j++) data[i * n + j] = ((float)i * (float)j) / (float)(n + 1);
}

/* correlation.cpp:35-87.  Float and double steps as in the reference:
 * the mean divides by (float)FLOAT_N; the variance by the double FLOAT_N,
 * rounded back to float; sqrt of the float value; eps compared in double;
 * the standardisation divides by the double sqrt(FLOAT_N), then by the
 * float standard deviation.  Unit diagonal. */
void orc_correlation_host(float* data, float* mean, float* stddev, float* symmat, idx_t n) {
  const idx_t ld = n + 1;
  for(idx_t j = 1; j <= n; j++) {
    mean[j] = 0.0f;
    for(idx_t i = 1; i <= n; i++) mean[j] += data[i * ld + j];
    mean[j] /= (float)kCorrFloatN;
  }
  for(idx_t j = 1; j <= n; j++) {
    stddev[j] = 0.0f;
    for(idx_t i = 1; i <= n; i++) {
      const float c = data[i * ld + j] - mean[j];
      stddev[j] += c * c;
    }
    stddev[j] = (float)((double)stddev[j] / kCorrFloatN);
    stddev[j] = (float)sqrt((double)stddev[j]);
    stddev[j] = (double)stddev[j] <= kCorrEps ? 1.0f : stddev[j];
  }
  const double root_n = sqrt(kCorrFloatN);
  for(idx_t i = 1; i <= n; i++)
    for(idx_t j = 1; j <= n; j++) {
      float v = data[i * ld + j] - mean[j];
      v = (float)((double)v / root_n);
      data[i * ld + j] = v / stddev[j];
    }
#pragma omp parallel for schedule(dynamic, 4)
  for(idx_t j1 = 1; j1 <= n - 1; j1++) {
    symmat[j1 * ld + j1] = 1.0f;
    for(idx_t j2 = j1 + 1; j2 <= n; j2++) {
      float acc = 0.0f;
      for(idx_t i = 1; i <= n; i++) acc += data[i * ld + j1] * data[i * ld + j2];
      symmat[j1 * ld + j2] = acc;
      symmat[j2 * ld + j1] = acc;
    }
  }
  if(n >= 1) symmat[n * ld + n] = 1.0f;
}

/* ------------------------------------------------------------ matmulchain -- */
/* runtime/matmulchain.cpp:11-30: c[i][j] = sum_k a[i][k] * b[k][j] with an
 * int running sum: each step adds the float product to the int sum in
 * float and truncates the result toward zero. */
void orc_matmulchain_product(const float* a, const float* b, float* c, idx_t n) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      int sum = 0;
      for(idx_t k = 0; k < n; k++) sum = (int)((float)sum + a[i * n + k] * b[k * n + j]);
      c[i * n + j] = (float)sum;
    }
}

/* --------------------------------------------------------- matrix-vector -- */
/* x[i] = i * M_PI in double, stored as float.  The reference's C++ builds see
 * glibc's M_PI (its 3.14159 fallback applies only where M_PI is undefined). */
static const double kPi = 3.14159265358979323846;

/* atax.cpp:20-30 */
void orc_atax_init(float* x, float* A, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    x[i] = (float)((double)i * kPi);
    for(idx_t j = 0; j < n; j++) A[i * n + j] = ((float)i * (float)j) / (float)n;
  }
}

/* atax.cpp:32-46: tmp[i] += A[i][j] x[j]; y[j] += A[i][j] tmp[i], row i by row i.
 * y and tmp are accumulated onto the caller's values (zeros in the reference). */
void orc_atax_host(const float* A, const float* x, float* y, float* tmp, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    for(idx_t j = 0; j < n; j++) tmp[i] += A[i * n + j] * x[j];
    for(idx_t j = 0; j < n; j++) y[j] += A[i * n + j] * tmp[i];
  }
}

/* bicg.cpp:20-35 */
void orc_bicg_init(float* A, float* p, float* r, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    r[i] = (float)((double)i * kPi);
    for(idx_t j = 0; j < n; j++) A[i * n + j] = ((float)i * (float)j) / (float)n;
  }
  for(idx_t i = 0; i < n; i++) p[i] = (float)((double)i * kPi);
}

/* bicg.cpp:37-48: s[j] += r[i] A[i][j]; q[i] += A[i][j] p[j]. */
void orc_bicg_host(const float* A, const float* r, float* s, const float* p, float* q, idx_t n) {
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) {
      s[j] += r[i] * A[i * n + j];
      q[i] += A[i * n + j] * p[j];
    }
}

/* mvt.cpp:16-28 */
void orc_mvt_init(float* a, float* x1, float* x2, float* y1, float* y2, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    x1[i] = 0.0f;
    x2[i] = 0.0f;
    y1[i] = 1.0f;
    y2[i] = 1.0f;
    for(idx_t j = 0; j < n; j++) a[i * n + j] = (float)((double)(i + j) + 1.0) / (float)n;
  }
}

/* mvt.cpp:30-42: x1 = x1 + A y1 and x2 = x2 + A y2 (both with A itself). */
void orc_mvt_host(const float* a, float* x1, float* x2, const float* y1, const float* y2, idx_t n) {
  for(idx_t i = 0; i < n; i++)
    for(idx_t j = 0; j < n; j++) x1[i] = x1[i] + a[i * n + j] * y1[j];
  for(idx_t k = 0; k < n; k++)
    for(idx_t l = 0; l < n; l++) x2[k] = x2[k] + a[k * n + l] * y2[l];
}

/* gesummv.cpp:30-41 */
void orc_gesummv_init(float* A, float* B, float* x, idx_t n) {
  for(idx_t i = 0; i < n; i++) {
    x[i] = 1.0f;
    for(idx_t j = 0; j < n; j++) {
      A[i * n + j] = 2.0f;
      B[i * n + j] = 3.0f;
    }
  }
}

/* gesummv.cpp:43-56, ALPHA = BETA = 1 (float constants). */
void orc_gesummv_host(const float* A, const float* B, const float* x, float* y, float* tmp, idx_t n) {
  const float alpha = 1.0f, beta = 1.0f;
  for(idx_t i = 0; i < n; i++) {
    tmp[i] = 0.0f;
    y[i] = 0.0f;
    for(idx_t j = 0; j < n; j++) {
      tmp[i] = A[i * n + j] * x[j] + tmp[i];
      y[i] = B[i * n + j] * x[j] + y[i];
    }
    y[i] = alpha * tmp[i] + beta * y[i];
  }
}

/* ---------------------------------------------------------- FP64 oracles -- */

/* out = alpha * op(A) op(B) + beta * C0 in double from FP32 operands,
 * op(X) = X (op 0) or X^T (op 1), row-major with leading dimensions.
 * C0 may be NULL (treated as zero).  `A2`,`B2` (may be NULL) add a second
 * product op(A2) op(B2) with the same ops (syr2k). */
void orc_gemm_f64(int op_a, int op_b, idx_t M, idx_t N, idx_t K, double alpha, const float* A, idx_t lda,
    const float* B, idx_t ldb, const float* A2, const float* B2, double beta, const float* C0, idx_t ldc,
    double* out, idx_t ldo) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < M; i++) {
    for(idx_t j = 0; j < N; j++) {
      double s = 0.0;
      for(idx_t k = 0; k < K; k++) {
        const double a = op_a ? A[k * lda + i] : A[i * lda + k];
        const double b = op_b ? B[j * ldb + k] : B[k * ldb + j];
        s += a * b;
        if(A2 && B2) {
          const double a2 = op_a ? A2[k * lda + i] : A2[i * lda + k];
          const double b2 = op_b ? B2[j * ldb + k] : B2[k * ldb + j];
          s += a2 * b2;
        }
      }
      out[i * ldo + j] = alpha * s + (C0 ? beta * (double)C0[i * ldc + j] : 0.0);
    }
  }
}

/* Same as orc_gemm_f64 with double operands (chained stages of 2mm/3mm). */
void orc_gemm_f64d(idx_t M, idx_t N, idx_t K, double alpha, const double* A, idx_t lda, const double* B, idx_t ldb,
    double beta, const double* C0, idx_t ldc, double* out, idx_t ldo) {
#pragma omp parallel for schedule(static)
  for(idx_t i = 0; i < M; i++)
    for(idx_t j = 0; j < N; j++) {
      double s = 0.0;
      for(idx_t k = 0; k < K; k++) s += A[i * lda + k] * B[k * ldb + j];
      out[i * ldo + j] = alpha * s + (C0 ? beta * C0[i * ldc + j] : 0.0);
    }
}

/* Normwise error of an FP32 result against an FP64 reference:
 *   max_rel  = max|C - R| / max|R|,   frob_rel = ||C - R||_F / ||R||_F.
 * Elementwise relative error max(|C-R|/|R|) over |R| > 0 also reported. */
void orc_error_norms(const float* C, const double* R, idx_t count, double* max_rel, double* frob_rel,
    double* max_elem_rel) {
  double max_err = 0, max_ref = 0, se = 0, sr = 0, mer = 0;
  for(idx_t i = 0; i < count; i++) {
    const double e = fabs((double)C[i] - R[i]);
    const double r = fabs(R[i]);
    if(e > max_err || e != e) max_err = e;
    if(r > max_ref) max_ref = r;
    se += e * e;
    sr += r * r;
    if(r > 0 && e / r > mer) mer = e / r;
  }
  if(max_rel) *max_rel = max_ref > 0 ? max_err / max_ref : max_err;
  if(frob_rel) *frob_rel = sr > 0 ? sqrt(se / sr) : sqrt(se);
  if(max_elem_rel) *max_elem_rel = mer;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
