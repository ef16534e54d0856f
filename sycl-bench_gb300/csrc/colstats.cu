// Column statistics and column normalisation for the covariance and
// correlation benchmarks (polybench/covariance.cpp, polybench/correlation.cpp):
// the passes that prepare the data matrix before its X^T.X contraction.
//
// The reference gives one work-item per column and walks the rows
// sequentially through global memory (covariance.cpp:84-96,
// correlation.cpp:111-142).  Here a column reduction is two launches:
//   * partial pass: a CTA of 8 warps owns 32 adjacent columns and one chunk
//     of rows; lane j of every warp reads column j (a warp reads 128
//     contiguous bytes of a row), each thread keeps eight independent loads
//     in flight, and the 8 warps are combined in shared memory into one
//     partial sum per (chunk, column);
//   * final pass: one thread per column adds its chunks' partials in chunk
//     order and applies the division (and, for standard deviations, the
//     square root and the eps clamp).
// The chunk count is chosen so that about four CTAs per SM stream the
// matrix; the result does not depend on the launch beyond that fixed
// summation tree (same inputs and shape, same bits).  All arithmetic is FP32.
#include "gbpoly_internal.cuh"

namespace gbpoly {
namespace {

constexpr int kColsPerBlock = 32;
constexpr int kWarps = 8;

// sum over rows [r0, r1) of f(X[r][j]) for this thread's column j, rows
// warp, warp + 8, ... of the chunk; eight loads in flight.
template <bool CENTERED>
__device__ __forceinline__ float column_chunk_sum(const float* __restrict__ col, int64_t ldx, int r0, int r1, int warp,
    float m) {
  constexpr int kLoads = 8;
  float a[kLoads];
#pragma unroll
  for(int k = 0; k < kLoads; ++k) a[k] = 0.f;
  int r = r0 + warp;
  for(; r + (kLoads - 1) * kWarps < r1; r += kLoads * kWarps) {
    float v[kLoads];
#pragma unroll
    for(int k = 0; k < kLoads; ++k) v[k] = col[int64_t(r + k * kWarps) * ldx];
#pragma unroll
    for(int k = 0; k < kLoads; ++k) {
      if constexpr(CENTERED) {
        const float c = v[k] - m;
        a[k] = fmaf(c, c, a[k]);
      } else {
        a[k] += v[k];
      }
    }
  }
  for(; r < r1; r += kWarps) {
    float v = col[int64_t(r) * ldx];
    if constexpr(CENTERED) {
      v -= m;
      a[0] = fmaf(v, v, a[0]);
    } else {
      a[0] += v;
    }
  }
  return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}

// partial[chunk][j] = sum over the chunk's rows of X[r][j] (or (X[r][j] - mean[j])^2).
template <bool CENTERED>
__global__ void __launch_bounds__(kWarps * 32) column_partial_kernel(const float* __restrict__ X, int64_t ldx, int rows,
    int cols, int rows_per_chunk, const float* __restrict__ mean, float* __restrict__ partial) {
  __shared__ float red[kWarps][kColsPerBlock + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = blockIdx.x * kColsPerBlock + lane;
  const int r0 = blockIdx.y * rows_per_chunk, r1 = min(rows, r0 + rows_per_chunk);
  float s = 0.f;
  if(j < cols) s = column_chunk_sum<CENTERED>(X + j, ldx, r0, r1, warp, CENTERED ? mean[j] : 0.f);
  red[warp][lane] = s;
  __syncthreads();
  if(warp == 0 && j < cols) {
    float t = red[0][lane];
#pragma unroll
    for(int w = 1; w < kWarps; ++w) t += red[w][lane];
    partial[int64_t(blockIdx.y) * cols + j] = t;
  }
}

// out[j] = (sum of the chunks' partials) / divisor; for standard deviations
// then sqrt, and 1 where the result is <= eps.
template <bool STDDEV>
__global__ void column_final_kernel(const float* __restrict__ partial, int chunks, int cols, float divisor, float eps,
    float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if(j >= cols) return;
  float s = 0.f;
  for(int c = 0; c < chunks; ++c) s += partial[int64_t(c) * cols + j];
  s = s / divisor;
  if constexpr(STDDEV) {
    s = sqrtf(s);
    s = s <= eps ? 1.f : s;
  }
  out[j] = s;
}

// Y[r][j] = X[r][j] - mean[j], or ((X[r][j] - mean[j]) / scale_div) / stddev[j].
template <bool SCALED>
__global__ void __launch_bounds__(256) center_columns_kernel(const float* X, int64_t ldx, int rows, int cols,
    const float* __restrict__ mean, const float* __restrict__ stddev, float scale_div, float* Y, int64_t ldy,
    int rows_per_block) {
  const int j = blockIdx.x * 32 + (threadIdx.x & 31);
  if(j >= cols) return;
  const float m = mean[j];
  const float sd = SCALED ? stddev[j] : 1.f;
  const int r0 = blockIdx.y * rows_per_block, r1 = min(rows, r0 + rows_per_block);
  // eight rows per batch, all loaded before the first store (Y may be X, so a
  // load could not otherwise move above the previous store)
  constexpr int kBatch = 8;
  for(int rb = r0 + (threadIdx.x >> 5); rb < r1; rb += 8 * kBatch) {
    float v[kBatch];
#pragma unroll
    for(int k = 0; k < kBatch; ++k) {
      const int r = rb + 8 * k;
      v[k] = r < r1 ? X[int64_t(r) * ldx + j] : 0.f;
    }
#pragma unroll
    for(int k = 0; k < kBatch; ++k) {
      const int r = rb + 8 * k;
      float y = v[k] - m;
      if constexpr(SCALED) y = (y / scale_div) / sd;
      if(r < r1) Y[int64_t(r) * ldy + j] = y;
    }
  }
}

__global__ void set_diagonal_kernel(int64_t n, float value, float* C, int64_t ldc) {
  for(int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    C[i * ldc + i] = value;
}

gbpoly_status check_block(const char* name, const void* p, int64_t rows, int64_t cols, int64_t ld) {
  if(rows > 0 && cols > 0) {
    if(!p) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": null pointer");
    if(ld < cols) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": leading dimension smaller than columns");
  }
  return GBPOLY_OK;
}

gbpoly_status check_args(gbpoly_ctx* ctx, int64_t rows, int64_t cols) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  if(rows < 0 || cols < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  if(rows >= (1ll << 31) || cols >= (1ll << 31)) return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large");
  return GBPOLY_OK;
}

// Column reduction: partial pass into the context's stats scratch, final pass into out.
template <bool STDDEV>
gbpoly_status column_reduce(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx, const float* mean,
    float divisor, float eps, float* out) {
  if(cols == 0) return GBPOLY_OK;
  const int col_blocks = int((cols + kColsPerBlock - 1) / kColsPerBlock);
  // about four CTAs per SM, at least 64 rows per chunk
  const int64_t want = std::max<int64_t>(1, (4ll * std::max(ctx->sm_count, 1) + col_blocks - 1) / col_blocks);
  const int64_t chunks = std::max<int64_t>(1, std::min<int64_t>(want, (rows + 63) / 64));
  const int rows_per_chunk = int((rows + chunks - 1) / chunks);
  gbpoly_status st = ensure_scratch(ctx, ctx->stats, size_t(chunks) * size_t(cols) * sizeof(float), "column scratch");
  if(st != GBPOLY_OK) return st;
  float* partial = static_cast<float*>(ctx->stats.ptr);
  {
    ProfileScope prof(ctx, STDDEV ? "column_sumsq" : "column_sum");
    column_partial_kernel<STDDEV><<<dim3(unsigned(col_blocks), unsigned(chunks)), kWarps * 32, 0, ctx->stream>>>(
        X, ldx, int(rows), int(cols), std::max(rows_per_chunk, 1), mean, partial);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  ProfileScope prof(ctx, STDDEV ? "column_stddev_final" : "column_mean_final");
  column_final_kernel<STDDEV><<<unsigned((cols + 255) / 256), 256, 0, ctx->stream>>>(partial, int(rows > 0 ? chunks : 0),
      int(cols), divisor, eps, out);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

}  // namespace
}  // namespace gbpoly

using namespace gbpoly;

extern "C" {

gbpoly_status gbpoly_column_mean_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    float divisor, float* mean) {
  gbpoly_status st = check_args(ctx, rows, cols);
  if(st != GBPOLY_OK) return st;
  if((st = check_block("X", X, rows, cols, ldx)) != GBPOLY_OK) return st;
  if(cols > 0 && !mean) return fail(GBPOLY_ERR_INVALID, "mean: null pointer");
  return column_reduce<false>(ctx, rows, cols, X, ldx, nullptr, divisor, 0.f, mean);
}

gbpoly_status gbpoly_column_stddev_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    const float* mean, float divisor, float eps, float* stddev) {
  gbpoly_status st = check_args(ctx, rows, cols);
  if(st != GBPOLY_OK) return st;
  if((st = check_block("X", X, rows, cols, ldx)) != GBPOLY_OK) return st;
  if(cols > 0 && (!mean || !stddev)) return fail(GBPOLY_ERR_INVALID, "mean/stddev: null pointer");
  return column_reduce<true>(ctx, rows, cols, X, ldx, mean, divisor, eps, stddev);
}

gbpoly_status gbpoly_center_columns_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* X, int64_t ldx,
    const float* mean, const float* stddev, float scale_div, float* Y, int64_t ldy) {
  gbpoly_status st = check_args(ctx, rows, cols);
  if(st != GBPOLY_OK) return st;
  if((st = check_block("X", X, rows, cols, ldx)) != GBPOLY_OK) return st;
  if((st = check_block("Y", Y, rows, cols, ldy)) != GBPOLY_OK) return st;
  if(cols > 0 && !mean) return fail(GBPOLY_ERR_INVALID, "mean: null pointer");
  if(X == Y && ldx != ldy) return fail(GBPOLY_ERR_INVALID, "in-place centring needs ldy == ldx");
  if(rows == 0 || cols == 0) return GBPOLY_OK;
  constexpr int kRowsPerBlock = 64;
  const dim3 grid(unsigned((cols + 31) / 32), unsigned((rows + kRowsPerBlock - 1) / kRowsPerBlock));
  if(grid.y > 65535u) return fail(GBPOLY_ERR_UNSUPPORTED, "too many rows");
  ProfileScope prof(ctx, stddev ? "normalize_columns" : "center_columns");
  if(stddev)
    center_columns_kernel<true><<<grid, 256, 0, ctx->stream>>>(X, ldx, int(rows), int(cols), mean, stddev, scale_div, Y,
        ldy, kRowsPerBlock);
  else
    center_columns_kernel<false><<<grid, 256, 0, ctx->stream>>>(X, ldx, int(rows), int(cols), mean, nullptr, 1.f, Y,
        ldy, kRowsPerBlock);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

gbpoly_status gbpoly_covariance_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t rows, int64_t cols, const float* X,
    int64_t ldx, const float* mean, const float* stddev, float scale_div, float* C, int64_t ldc) {
  gbpoly_status st = check_args(ctx, rows, cols);
  if(st != GBPOLY_OK) return st;
  if((st = check_block("X", X, rows, cols, ldx)) != GBPOLY_OK) return st;
  if((st = check_block("C", C, cols, cols, ldc)) != GBPOLY_OK) return st;
  if(cols > 0 && !mean) return fail(GBPOLY_ERR_INVALID, "mean: null pointer");
  if(cols == 0) return GBPOLY_OK;
  GemmF32Args a{};
  a.M = cols, a.N = cols, a.K = rows, a.alpha = 1.f, a.beta = 0.f, a.op_a = GBPOLY_OP_T, a.op_b = GBPOLY_OP_N;
  a.C = C, a.ldc = ldc;
  const bool split_form = prec == GBPOLY_PREC_TF32 || prec == GBPOLY_PREC_BF16X3 || prec == GBPOLY_PREC_TF32X3 ||
                          prec == GBPOLY_PREC_BF16X6 || prec == GBPOLY_PREC_FP16X3;
  if(split_form && rows > 0) {
    // centred in the split pass: X itself is both operands
    a.A = X, a.lda = ldx, a.B = X, a.ldb = ldx;
    a.xf = RowXform{mean, stddev, scale_div};
    return launch_gemm_tensor(ctx, prec, a);
  }
  if(prec != GBPOLY_PREC_FP32 && prec != GBPOLY_PREC_FP8 && !split_form)
    return fail(GBPOLY_ERR_INVALID, "unknown precision");
  // a centred copy with 16-byte-aligned rows, then the contraction
  const int64_t ldy = (cols + 3) / 4 * 4;
  if((st = ensure_scratch(ctx, ctx->centred, size_t(std::max<int64_t>(rows, 1)) * size_t(ldy) * 4 + 256,
          "centred copy")) != GBPOLY_OK)
    return st;
  float* Y = static_cast<float*>(ctx->centred.ptr);
  if((st = gbpoly_center_columns_f32(ctx, rows, cols, X, ldx, mean, stddev, scale_div, Y, ldy)) != GBPOLY_OK)
    return st;
  a.A = Y, a.lda = ldy, a.B = Y, a.ldb = ldy;
  return prec == GBPOLY_PREC_FP32 ? launch_gemm_f32_simt(ctx, a) : launch_gemm_tensor(ctx, prec, a);
}

gbpoly_status gbpoly_set_diagonal_f32(gbpoly_ctx* ctx, int64_t n, float value, float* C, int64_t ldc) {
  gbpoly_status st = check_args(ctx, n, n);
  if(st != GBPOLY_OK) return st;
  if((st = check_block("C", C, n, n, ldc)) != GBPOLY_OK) return st;
  if(n == 0) return GBPOLY_OK;
  ProfileScope prof(ctx, "set_diagonal");
  set_diagonal_kernel<<<unsigned(std::min<int64_t>((n + 255) / 256, 4096)), 256, 0, ctx->stream>>>(n, value, C, ldc);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

}  // extern "C"
