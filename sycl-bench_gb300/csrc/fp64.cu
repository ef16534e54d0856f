// FP64 on the GPU: the oracle DGEMM for error norms at sizes the host cannot
// finish, the double variants of the benchmarks, and the error-norm
// reduction of an FP32 result against an FP64 reference.
#include <cmath>

#include "gbpoly_internal.cuh"
#include "tiled_gemm.cuh"

namespace gbpoly {
namespace {

__global__ void convert_f32_f64_kernel(const float* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for(int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[i] = static_cast<double>(src[i]);
}

// Per-block partial statistics of e = |C - R|, r = |R| over a rows x cols window:
//   [0] max e, [1] max r, [2] sum e^2, [3] sum r^2, [4] max e/r (r > 0), [5] count of non-finite e
constexpr int kStats = 6;
constexpr int kNormThreads = 256;

__device__ __forceinline__ void combine(double* a, const double* b) {
  a[0] = fmax(a[0], b[0]);
  a[1] = fmax(a[1], b[1]);
  a[2] += b[2];
  a[3] += b[3];
  a[4] = fmax(a[4], b[4]);
  a[5] += b[5];
}

__device__ void block_reduce(double (&v)[kStats], double* out) {
  __shared__ double sh[kNormThreads / 32][kStats];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for(int off = 16; off > 0; off >>= 1) {
    double o[kStats];
#pragma unroll
    for(int s = 0; s < kStats; ++s) o[s] = __shfl_down_sync(0xffffffffu, v[s], off);
    combine(v, o);
  }
  if(lane == 0)
#pragma unroll
    for(int s = 0; s < kStats; ++s) sh[warp][s] = v[s];
  __syncthreads();
  if(threadIdx.x == 0) {
    for(int w = 1; w < kNormThreads / 32; ++w) combine(sh[0], sh[w]);
#pragma unroll
    for(int s = 0; s < kStats; ++s) out[s] = sh[0][s];
  }
}

__global__ void __launch_bounds__(kNormThreads) error_norms_partial_kernel(const float* __restrict__ C, int64_t ldc,
    const double* __restrict__ R, int64_t ldr, int64_t rows, int64_t cols, double* __restrict__ partial) {
  double v[kStats] = {0, 0, 0, 0, 0, 0};
  const int64_t total = rows * cols;
  for(int64_t idx = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; idx < total;
      idx += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = idx / cols, c = idx - r * cols;
    const double ref = R[r * ldr + c];
    const double e = fabs(static_cast<double>(C[r * ldc + c]) - ref);
    const double ar = fabs(ref);
    if(!isfinite(e)) {
      v[5] += 1;
      continue;
    }
    v[0] = fmax(v[0], e);
    v[1] = fmax(v[1], ar);
    v[2] += e * e;
    v[3] += ar * ar;
    if(ar > 0) v[4] = fmax(v[4], e / ar);
  }
  block_reduce(v, partial + blockIdx.x * kStats);
}

__global__ void __launch_bounds__(kNormThreads) error_norms_final_kernel(const double* __restrict__ partial,
    int nblocks, double* __restrict__ out) {
  double v[kStats] = {0, 0, 0, 0, 0, 0};
  for(int b = threadIdx.x; b < nblocks; b += blockDim.x) combine(v, partial + b * kStats);
  block_reduce(v, out);
}

}  // namespace
}  // namespace gbpoly

using namespace gbpoly;

namespace {
gbpoly_status check_mat(const char* name, const void* p, int64_t rows, int64_t cols, int64_t ld) {
  if(rows < 0 || cols < 0) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": negative dimension");
  if(rows > 0 && cols > 0) {
    if(!p) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": null pointer");
    if(ld < cols) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": leading dimension smaller than columns");
  }
  return GBPOLY_OK;
}

TiledOperand<double> opnd(const double* p, int64_t ld, gbpoly_op op) {
  return op == GBPOLY_OP_N ? TiledOperand<double>{p, ld, 1} : TiledOperand<double>{p, 1, ld};
}
}  // namespace

extern "C" {

gbpoly_status gbpoly_gemm_f64(gbpoly_ctx* ctx, gbpoly_op op_a, gbpoly_op op_b, int64_t M, int64_t N, int64_t K,
    double alpha, const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  if((op_a != GBPOLY_OP_N && op_a != GBPOLY_OP_T) || (op_b != GBPOLY_OP_N && op_b != GBPOLY_OP_T))
    return fail(GBPOLY_ERR_INVALID, "bad operand op");
  if(M < 0 || N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  gbpoly_status st;
  if((st = check_mat("A", A, op_a == GBPOLY_OP_N ? M : K, op_a == GBPOLY_OP_N ? K : M, lda)) != GBPOLY_OK) return st;
  if((st = check_mat("B", B, op_b == GBPOLY_OP_N ? K : N, op_b == GBPOLY_OP_N ? N : K, ldb)) != GBPOLY_OK) return st;
  if((st = check_mat("C", C, M, N, ldc)) != GBPOLY_OK) return st;
  // op(B)[k][n] is addressed as TiledOperand over (n, k)
  TiledOperand<double> ob = op_b == GBPOLY_OP_N ? TiledOperand<double>{B, 1, ldb} : TiledOperand<double>{B, ldb, 1};
  // op(B) = op(A)^T on the same matrix (syrk's A.A^T, X^T.X): symmetric, lower triangle of tiles + mirror
  const bool symmetric = A == B && lda == ldb && M == N && op_a != op_b;
  return launch_tiled_gemm<double>(ctx, M, N, K, alpha, opnd(A, lda, op_a), ob, false, {}, {}, beta, C, ldc,
      symmetric);
}

gbpoly_status gbpoly_syrk_f64(gbpoly_ctx* ctx, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
    double beta, double* C, int64_t ldc) {
  return gbpoly_gemm_f64(ctx, GBPOLY_OP_N, GBPOLY_OP_T, N, N, K, alpha, A, lda, A, lda, beta, C, ldc);
}

gbpoly_status gbpoly_syr2k_f64(gbpoly_ctx* ctx, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
    const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  gbpoly_status st;
  if(N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  if((st = check_mat("A", A, N, K, lda)) != GBPOLY_OK) return st;
  if((st = check_mat("B", B, N, K, ldb)) != GBPOLY_OK) return st;
  if((st = check_mat("C", C, N, N, ldc)) != GBPOLY_OK) return st;
  return launch_tiled_gemm<double>(ctx, N, N, K, alpha, TiledOperand<double>{A, lda, 1},
      TiledOperand<double>{B, ldb, 1}, true, TiledOperand<double>{B, ldb, 1}, TiledOperand<double>{A, lda, 1}, beta,
      C, ldc, true);  // symmetric: lower triangle of tiles + mirror
}

gbpoly_status gbpoly_convert_f32_f64(gbpoly_ctx* ctx, const float* src, double* dst, int64_t count) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  if(count < 0) return fail(GBPOLY_ERR_INVALID, "negative count");
  if(count == 0) return GBPOLY_OK;
  if(!src || !dst) return fail(GBPOLY_ERR_INVALID, "null pointer");
  const int64_t blocks = std::min<int64_t>((count + 255) / 256, int64_t(ctx->sm_count) * 16);
  ProfileScope prof(ctx, "convert_f32_f64");
  convert_f32_f64_kernel<<<static_cast<unsigned>(blocks), 256, 0, ctx->stream>>>(src, dst, count);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

gbpoly_status gbpoly_error_norms(gbpoly_ctx* ctx, const float* C, int64_t ldc, const double* R, int64_t ldr,
    int64_t rows, int64_t cols, double* max_rel, double* frob_rel, double* max_elem_rel) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  gbpoly_status st;
  if((st = check_mat("C", C, rows, cols, ldc)) != GBPOLY_OK) return st;
  if((st = check_mat("R", R, rows, cols, ldr)) != GBPOLY_OK) return st;
  double h[kStats] = {0, 0, 0, 0, 0, 0};
  if(rows > 0 && cols > 0) {
    const int blocks = ctx->sm_count * 4;
    if((st = ensure_workspace(ctx, size_t(blocks + 1) * kStats * sizeof(double))) != GBPOLY_OK) return st;
    double* partial = static_cast<double*>(ctx->ws.ptr);
    double* out = partial + size_t(blocks) * kStats;
    ProfileScope prof(ctx, "error_norms");
    error_norms_partial_kernel<<<blocks, kNormThreads, 0, ctx->stream>>>(C, ldc, R, ldr, rows, cols, partial);
    GBPOLY_CUDA_TRY(cudaGetLastError());
    error_norms_final_kernel<<<1, kNormThreads, 0, ctx->stream>>>(partial, blocks, out);
    GBPOLY_CUDA_TRY(cudaGetLastError());
    GBPOLY_CUDA_TRY(cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    GBPOLY_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  }
  const double inf = HUGE_VAL;
  const bool bad = h[5] > 0;
  if(max_rel) *max_rel = bad ? inf : (h[1] > 0 ? h[0] / h[1] : h[0]);
  if(frob_rel) *frob_rel = bad ? inf : (h[3] > 0 ? std::sqrt(h[2] / h[3]) : std::sqrt(h[2]));
  if(max_elem_rel) *max_elem_rel = bad ? inf : h[4];
  return GBPOLY_OK;
}

}  // extern "C"
