// Host-buffer contraction: C <- alpha op(A) op(B) + beta C with A, B, C in
// host memory, the copies pipelined with the computation.
//
// The link between host and device memory is the limit of this call (on a
// GB300 machine about 211 GB/s host->device and 193 GB/s device->host, each a
// little lower when both run), so the work is split into row panels of C:
// B goes over first and is split once; then for every panel the copy
// stream brings its rows of A (and C when beta != 0), the context stream
// splits them and runs the panel's contraction, and a second copy stream
// returns the panel of C while the next panel's rows travel the other way.
// Device staging (operands and term panels) stays allocated in the context.
#include <algorithm>
#include <cstring>

#include "gbpoly_internal.cuh"

namespace gbpoly {
namespace {

gbpoly_status ensure_buffer(void*& p, size_t& have, size_t need) {
  if(have >= need) return GBPOLY_OK;
  if(p) cudaFree(p);
  p = nullptr;
  have = 0;
  GBPOLY_CUDA_TRY(cudaMalloc(&p, need));
  have = need;
  return GBPOLY_OK;
}

gbpoly_status ensure_streams(gbpoly_ctx* ctx) {
  if(!ctx->h2d_stream) GBPOLY_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->h2d_stream, cudaStreamNonBlocking));
  if(!ctx->d2h_stream) GBPOLY_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->d2h_stream, cudaStreamNonBlocking));
  return GBPOLY_OK;
}

// rows x cols floats between a host matrix with leading dimension ld and a
// compact device matrix
gbpoly_status copy_rows(void* dst, size_t dpitch, const void* src, size_t spitch, int64_t rows, int64_t cols,
    cudaMemcpyKind kind, cudaStream_t s) {
  if(rows <= 0 || cols <= 0) return GBPOLY_OK;
  GBPOLY_CUDA_TRY(cudaMemcpy2DAsync(dst, dpitch, src, spitch, size_t(cols) * 4, size_t(rows), kind, s));
  return GBPOLY_OK;
}

}  // namespace
}  // namespace gbpoly

using namespace gbpoly;

extern "C" gbpoly_status gbpoly_gemm_f32_host(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op op_a, gbpoly_op op_b,
    int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb,
    float beta, float* C, int64_t ldc) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  if((op_a != GBPOLY_OP_N && op_a != GBPOLY_OP_T) || (op_b != GBPOLY_OP_N && op_b != GBPOLY_OP_T))
    return fail(GBPOLY_ERR_INVALID, "bad operand op");
  if(M < 0 || N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  const int64_t ar = op_a == GBPOLY_OP_N ? M : K, ac = op_a == GBPOLY_OP_N ? K : M;
  const int64_t br = op_b == GBPOLY_OP_N ? K : N, bc = op_b == GBPOLY_OP_N ? N : K;
  if((ar > 0 && ac > 0 && (!A || lda < ac)) || (br > 0 && bc > 0 && (!B || ldb < bc)) ||
      (M > 0 && N > 0 && (!C || ldc < N)))
    return fail(GBPOLY_ERR_INVALID, "null matrix or leading dimension smaller than its columns");
  if(M == 0 || N == 0) return GBPOLY_OK;
  gbpoly_status st;
  if((st = ensure_streams(ctx)) != GBPOLY_OK) return st;
  // device copies: compact (ld = columns)
  if((st = ensure_buffer(ctx->stage_a, ctx->stage_a_bytes, size_t(std::max<int64_t>(ar * ac, 1)) * 4)) != GBPOLY_OK)
    return st;
  if((st = ensure_buffer(ctx->stage_b, ctx->stage_b_bytes, size_t(std::max<int64_t>(br * bc, 1)) * 4)) != GBPOLY_OK)
    return st;
  if((st = ensure_buffer(ctx->stage_c, ctx->stage_c_bytes, size_t(M) * N * 4)) != GBPOLY_OK) return st;
  float* dA = static_cast<float*>(ctx->stage_a);
  float* dB = static_cast<float*>(ctx->stage_b);
  float* dC = static_cast<float*>(ctx->stage_c);

  // Row panels of C (and of op(A) when A is stored row by row), at most 16 of
  // at least 512 rows (a multiple of the 256-row tiles of CTA pairs): the
  // copies are the bound, and what stays exposed after the last input copy
  // is one panel's contraction and read-back.
  const bool pipelined = op_a == GBPOLY_OP_N;
  int panels = pipelined ? int(std::min<int64_t>(16, std::max<int64_t>(1, M / 512))) : 1;
  const int64_t rows_per = ((M + panels - 1) / panels + 255) / 256 * 256;
  panels = int((M + rows_per - 1) / rows_per);

  cudaEvent_t ev_in = nullptr, ev_done = nullptr;
  GBPOLY_CUDA_TRY(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
  GBPOLY_CUDA_TRY(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming));
  struct Guard {
    cudaEvent_t a, b;
    ~Guard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } guard{ev_in, ev_done};

  // the copy streams start after everything already queued on the context stream
  GBPOLY_CUDA_TRY(cudaEventRecord(ev_in, ctx->stream));
  GBPOLY_CUDA_TRY(cudaStreamWaitEvent(ctx->h2d_stream, ev_in, 0));
  GBPOLY_CUDA_TRY(cudaStreamWaitEvent(ctx->d2h_stream, ev_in, 0));

  // B (all of it), then A whole when it is not split in row panels
  if((st = copy_rows(dB, size_t(bc) * 4, B, size_t(ldb) * 4, br, bc, cudaMemcpyHostToDevice, ctx->h2d_stream)) != GBPOLY_OK)
    return st;
  if(!pipelined &&
      (st = copy_rows(dA, size_t(ac) * 4, A, size_t(lda) * 4, ar, ac, cudaMemcpyHostToDevice, ctx->h2d_stream)) != GBPOLY_OK)
    return st;
  TensorPlan plan;
  if(prec != GBPOLY_PREC_FP32) {
    if((st = tensor_plan(ctx, prec, op_a, op_b, M, N, K, &plan)) != GBPOLY_OK) return st;
  }
  for(int p = 0; p < panels; ++p) {
    const int64_t r0 = p * rows_per, rows = std::min<int64_t>(rows_per, M - r0);
    if(pipelined &&
        (st = copy_rows(dA + r0 * K, size_t(K) * 4, A + r0 * lda, size_t(lda) * 4, rows, K, cudaMemcpyHostToDevice,
             ctx->h2d_stream)) != GBPOLY_OK)
      return st;
    if(beta != 0.f &&
        (st = copy_rows(dC + r0 * N, size_t(N) * 4, C + r0 * ldc, size_t(ldc) * 4, rows, N, cudaMemcpyHostToDevice,
             ctx->h2d_stream)) != GBPOLY_OK)
      return st;
    GBPOLY_CUDA_TRY(cudaEventRecord(ev_in, ctx->h2d_stream));
    GBPOLY_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_in, 0));
    GemmF32Args a{};
    a.M = pipelined ? rows : M, a.N = N, a.K = K, a.alpha = alpha, a.beta = beta, a.op_a = op_a, a.op_b = op_b;
    a.A = pipelined ? dA + r0 * K : dA, a.lda = ac, a.B = dB, a.ldb = bc, a.C = dC + r0 * N, a.ldc = N;
    if(prec == GBPOLY_PREC_FP32) {
      // the K split of the whole call on equally aligned device operands
      // (operands the TMA kernel cannot read are not split), so the panels
      // give the device-buffer call's bits
      const bool tma_like = ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) == 0 &&
                            lda % 4 == 0 && ldb % 4 == 0;
      a.ksplit = tma_like ? fp32_split_k_count(ctx->sm_count, M, N, K) : 1;
      st = launch_gemm_f32_simt(ctx, a);
    }
    else
      st = tensor_plan_panel(ctx, plan, a, p == 0, r0);
    if(st != GBPOLY_OK) return st;
    GBPOLY_CUDA_TRY(cudaEventRecord(ev_done, ctx->stream));
    GBPOLY_CUDA_TRY(cudaStreamWaitEvent(ctx->d2h_stream, ev_done, 0));
    if((st = copy_rows(C + r0 * ldc, size_t(ldc) * 4, dC + r0 * N, size_t(N) * 4, rows, N, cudaMemcpyDeviceToHost,
            ctx->d2h_stream)) != GBPOLY_OK)
      return st;
  }
  // later work on the context stream (and gbpoly_synchronize) waits for the returned panels
  GBPOLY_CUDA_TRY(cudaEventRecord(ev_done, ctx->d2h_stream));
  GBPOLY_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ev_done, 0));
  return GBPOLY_OK;
}
