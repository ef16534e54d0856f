// Simple tiled GEMM over general strides, templated on the element type.
//
// Used where TMA cannot describe an operand (FP32 operands whose base or
// leading dimension is not a multiple of 16 bytes) and as the FP64 DGEMM
// (the FP64 oracle and the double variants of the benchmarks; GB300's FP64
// rate is low enough that this SIMT tiling is not the limit).
//   op(X)[r][k] = X[r * s_r + k * s_k]
//   C[m][n] = alpha * (sum_k op(A)[m][k] op(B)[k][n]  [+ op(A2) op(B2)]) + beta * C[m][n]
// 64x64 tile of C per 256-thread CTA, 4x4 per thread, BK = 16.  beta == 0
// does not read C.  `lower` (symmetric products, M == N): only tiles on or
// below the diagonal compute; a tile below it also stores its transpose.
#pragma once
#include "gbpoly_internal.cuh"

namespace gbpoly {

template <typename T>
struct TiledOperand {
  const T* p;
  int64_t s_r, s_k;
};

template <typename T>
__global__ void __launch_bounds__(256) tiled_gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha,
    TiledOperand<T> a, TiledOperand<T> b, bool dual, TiledOperand<T> a2, TiledOperand<T> b2, T beta,
    T* __restrict__ C, int64_t ldc, bool lower) {
  __shared__ T As[16][64 + 1];
  __shared__ T Bs[16][64 + 1];
  if(lower && blockIdx.x > blockIdx.y) return;  // strictly above the diagonal: the mirror of another tile
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = static_cast<int64_t>(blockIdx.y) * 64, n0 = static_cast<int64_t>(blockIdx.x) * 64;
  T acc[4][4];
#pragma unroll
  for(int i = 0; i < 4; ++i)
#pragma unroll
    for(int j = 0; j < 4; ++j) acc[i][j] = T(0);
  const int passes = dual ? 2 : 1;
  for(int p = 0; p < passes; ++p) {
    const TiledOperand<T> oa = p ? a2 : a;
    const TiledOperand<T> ob = p ? b2 : b;
    for(int64_t k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
      for(int e = 0; e < 4; ++e) {
        const int idx = tid + e * 256;  // 0..1023 over a 64 x 16 tile
        // rows fastest when the operand is contiguous along rows, else k fastest
        const int r = (oa.s_r == 1) ? (idx & 63) : (idx >> 4);
        const int kk = (oa.s_r == 1) ? (idx >> 6) : (idx & 15);
        const int64_t gm = m0 + r, gk = k0 + kk;
        As[kk][r] = (gm < M && gk < K) ? oa.p[gm * oa.s_r + gk * oa.s_k] : T(0);
        const int rb = (ob.s_r == 1) ? (idx & 63) : (idx >> 4);
        const int kb = (ob.s_r == 1) ? (idx >> 6) : (idx & 15);
        const int64_t gn = n0 + rb, gkb = k0 + kb;
        Bs[kb][rb] = (gn < N && gkb < K) ? ob.p[gn * ob.s_r + gkb * ob.s_k] : T(0);
      }
      __syncthreads();
#pragma unroll
      for(int kk = 0; kk < 16; ++kk)
#pragma unroll
        for(int i = 0; i < 4; ++i)
#pragma unroll
          for(int j = 0; j < 4; ++j) acc[i][j] = fma(As[kk][ty * 4 + i], Bs[kk][tx + 16 * j], acc[i][j]);
      __syncthreads();
    }
  }
  // C values are loaded before the first store (a load cannot move above a
  // store that may alias it)
  T cv[4][4];
#pragma unroll
  for(int i = 0; i < 4; ++i)
#pragma unroll
    for(int j = 0; j < 4; ++j) {
      const int64_t m = m0 + ty * 4 + i, n = n0 + tx + 16 * j;
      cv[i][j] = (beta != T(0) && m < M && n < N) ? C[m * ldc + n] : T(0);
    }
#pragma unroll
  for(int i = 0; i < 4; ++i) {
    const int64_t m = m0 + ty * 4 + i;
    if(m >= M) continue;
#pragma unroll
    for(int j = 0; j < 4; ++j) {
      const int64_t n = n0 + tx + 16 * j;
      if(n < N) C[m * ldc + n] = fma(beta, cv[i][j], alpha * acc[i][j]);
    }
  }
  if(lower && blockIdx.x < blockIdx.y) {  // the transposed tile, C[n][m]
#pragma unroll
    for(int i = 0; i < 4; ++i)
#pragma unroll
      for(int j = 0; j < 4; ++j) {
        const int64_t m = m0 + ty * 4 + i, n = n0 + tx + 16 * j;
        cv[i][j] = (beta != T(0) && m < M && n < N) ? C[n * ldc + m] : T(0);
      }
#pragma unroll
    for(int i = 0; i < 4; ++i) {
      const int64_t m = m0 + ty * 4 + i;
      if(m >= M) continue;
#pragma unroll
      for(int j = 0; j < 4; ++j) {
        const int64_t n = n0 + tx + 16 * j;
        if(n < N) C[n * ldc + m] = fma(beta, cv[i][j], alpha * acc[i][j]);
      }
    }
  }
}

template <typename T>
gbpoly_status launch_tiled_gemm(gbpoly_ctx* ctx, int64_t M, int64_t N, int64_t K, T alpha, TiledOperand<T> a,
    TiledOperand<T> b, bool dual, TiledOperand<T> a2, TiledOperand<T> b2, T beta, T* C, int64_t ldc,
    bool lower = false) {
  if(M == 0 || N == 0) return GBPOLY_OK;
  const int64_t gx = (N + 63) / 64, gy = (M + 63) / 64;
  if(gy > 65535) return fail(GBPOLY_ERR_UNSUPPORTED, "matrix too tall for the tiled kernel grid");
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  ProfileScope prof(ctx, sizeof(T) == 8 ? "dgemm_tiled" : "sgemm_tiled");
  tiled_gemm_kernel<T><<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, a, b, dual, a2, b2, beta, C, ldc,
      lower && M == N);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

}  // namespace gbpoly
