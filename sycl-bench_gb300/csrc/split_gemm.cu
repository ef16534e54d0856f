// Tensor-core precision forms of the FP32 contraction (tcgen05, sm_103a).
//
// An FP32 operand x is split into T terms of a narrower type,
//     x ~= t0 + t1 (+ t2),  t0 = rn(x),  t1 = rn(x - t0),  t2 = rn(x - t0 - t1)
// (each difference is exact in FP32), and op(A).op(B) is accumulated in FP32
// in tensor memory from a subset of the term products:
//   form      type  terms  products                              bits kept
//   tf32      TF32  1      a0.b0                                 11
//   bf16x3    BF16  2      a0.b0 + a0.b1 + a1.b0                 ~16
//   tf32x3    TF32  2      a0.b0 + a0.b1 + a1.b0                 ~22-24
//   bf16x6    BF16  3      a0.b0 + a0.b1 + a1.b0 + a0.b2 + a1.b1 + a2.b0   ~24
// Two kernels per call:
//   * split_kernel (memory bound): writes the K-major term panels of an
//     operand into the context workspace (transposing through shared memory
//     when the operand is MN-major), K padded with zeros to the k-block;
//   * split_gemm_kernel: one 128 x BN tile of C per CTA, warp specialised:
//       warp 0     TMA producer: the term tiles of A (128 rows) and B (BN rows),
//                  128-byte rows (64 BF16 or 32 TF32 along K) with 128-byte
//                  swizzle, into a ring of STAGES shared-memory stages;
//       warp 1     allocates BN TMEM columns; one lane issues the products'
//                  tcgen05.mma (M=128, N=BN; K=16 BF16 or K=8 TF32) and
//                  commits each stage back to the producer;
//       warps 4-7  epilogue: tcgen05.ld of the accumulator (one TMEM lane
//                  quarter per warp), C = alpha*acc + beta*C.
//     syr2k's two products (A_i.B_j^T + B_i.A_j^T) alternate stage by stage
//     into the same accumulator.
// All mbarrier waits are bounded (gbpoly_internal.cuh).
#include <cuda_bf16.h>

#include "gbpoly_internal.cuh"
#include "umma.cuh"

namespace gbpoly {
namespace {

enum class Elem { BF16, TF32 };

template <Elem E, int TERMS, int NPROD, int BN_, int STAGES_>
struct Form {
  static constexpr Elem elem = E;
  static constexpr int terms = TERMS, nprod = NPROD, BM = 128, BN = BN_, STAGES = STAGES_;
  static constexpr int esz = E == Elem::BF16 ? 2 : 4;
  static constexpr int BK = 128 / esz;                 // elements per 128-byte row
  static constexpr int KMMA = E == Elem::BF16 ? 16 : 8; // K of one tcgen05.mma (32 bytes)
  static constexpr int A_TILE = BM * 128, B_TILE = BN * 128;
  static constexpr int STAGE = TERMS * (A_TILE + B_TILE);
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
  static constexpr uint32_t TMEM_COLS = BN;
  static constexpr uint32_t IDESC =
      umma::InstrDesc<BM, BN, E == Elem::BF16 ? umma::AbType::BF16 : umma::AbType::TF32>::value;
  static_assert(SMEM <= 232448, "shared memory");
};

using FormTF32 = Form<Elem::TF32, 1, 1, 256, 4>;
using FormBF16x3 = Form<Elem::BF16, 2, 3, 256, 2>;
using FormTF32x3 = Form<Elem::TF32, 2, 3, 256, 2>;
using FormBF16x6 = Form<Elem::BF16, 3, 6, 128, 2>;

// Term indices of product p: (0,0) (0,1) (1,0) (0,2) (1,1) (2,0)
__host__ __device__ constexpr int prod_a(int p) { return p == 2 ? 1 : (p == 4 ? 1 : (p == 5 ? 2 : 0)); }
__host__ __device__ constexpr int prod_b(int p) { return p == 1 ? 1 : (p == 3 ? 2 : (p == 4 ? 1 : 0)); }

// ---------------------------------------------------------------- rounding --
// Round to nearest even at TF32 precision (10 explicit mantissa bits); the
// low 13 bits become zero, which is what kind::tf32 reads.  Inf/NaN pass.
__device__ __forceinline__ float round_tf32(float x) {
  uint32_t u = __float_as_uint(x);
  if((u & 0x7f800000u) == 0x7f800000u) return x;
  u += 0xFFFu + ((u >> 13) & 1u);
  return __uint_as_float(u & 0xFFFFE000u);
}

template <Elem E>
struct Term;
template <>
struct Term<Elem::BF16> {
  using T = __nv_bfloat16;
  __device__ static T round(float x) { return __float2bfloat16_rn(x); }
  __device__ static float widen(T x) { return __bfloat162float(x); }
};
template <>
struct Term<Elem::TF32> {
  using T = float;
  __device__ static T round(float x) { return round_tf32(x); }
  __device__ static float widen(T x) { return x; }
};

// ------------------------------------------------------------- split pass --
// panel[t][r][k] (r < R, k < Kp) = term t of op(X)[r][k] for k < K, 0 beyond,
// op(X)[r][k] = X[r*ld + k] (k_major) or X[k*ld + r].  Panels are Kp-strided
// and `panel_stride` elements apart.
template <Elem E, int TERMS>
__global__ void __launch_bounds__(256) split_kernel(const float* __restrict__ X, int64_t ld, int k_major, int R, int K,
    int Kp, typename Term<E>::T* __restrict__ out, int64_t panel_stride) {
  using T = typename Term<E>::T;
  __shared__ float tile[64][65];
  const int tid = threadIdx.x;
  const int64_t r0 = int64_t(blockIdx.y) * 64, k0 = int64_t(blockIdx.x) * 64;
#pragma unroll
  for(int e = 0; e < 16; ++e) {
    const int idx = tid + e * 256;
    const int rr = k_major ? (idx >> 6) : (idx & 63);
    const int kk = k_major ? (idx & 63) : (idx >> 6);
    const int64_t r = r0 + rr, k = k0 + kk;
    float v = 0.f;
    if(r < R && k < K) v = k_major ? X[r * ld + k] : X[k * ld + r];
    tile[rr][kk] = v;
  }
  __syncthreads();
  const int rr = tid >> 2, kc = (tid & 3) * 16;
  const int64_t r = r0 + rr;
  if(r >= R) return;
  __align__(16) T t[TERMS][16];
#pragma unroll
  for(int i = 0; i < 16; ++i) {
    float rem = tile[rr][kc + i];
#pragma unroll
    for(int j = 0; j < TERMS; ++j) {
      t[j][i] = Term<E>::round(rem);
      rem -= Term<E>::widen(t[j][i]);
    }
  }
  constexpr int kVec = 16 * sizeof(T) / 16;  // uint4 per 16 elements
#pragma unroll
  for(int j = 0; j < TERMS; ++j) {
    uint4* dst = reinterpret_cast<uint4*>(out + j * panel_stride + r * Kp + k0 + kc);
#pragma unroll
    for(int v = 0; v < kVec; ++v) dst[v] = reinterpret_cast<const uint4*>(t[j])[v];
  }
}

// Tensor maps of one product pairing: left operand terms in 128-row boxes,
// right operand terms in BN-row boxes.
struct ProductMaps {
  CUtensorMap l[3], r[3];
};
struct GemmMaps {
  ProductMaps p[2];
};

__device__ __forceinline__ void tile_coords(int id, int tiles_m, int tiles_n, int& tile_m, int& tile_n) {
  constexpr int G = 16;
  const int per_group = G * tiles_n;
  const int group = id / per_group;
  const int first = group * G;
  const int gsz = min(tiles_m - first, G);
  const int r = id - group * per_group;
  tile_m = first + r % gsz;
  tile_n = r / gsz;
}

template <class F>
__global__ void __launch_bounds__(256, 1) split_gemm_kernel(const __grid_constant__ GemmMaps maps, int npair, int M,
    int N, int Kp, float alpha, float beta, float* __restrict__ C, int64_t ldc, int* err) {
  extern __shared__ __align__(1024) char smem_raw[];
  char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + F::STAGES * F::STAGE);
  uint64_t* empty = full + F::STAGES;
  uint64_t* accum = empty + F::STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_m = (M + F::BM - 1) / F::BM, tiles_n = (N + F::BN - 1) / F::BN;
  int tile_m, tile_n;
  tile_coords(blockIdx.x, tiles_m, tiles_n, tile_m, tile_n);
  const int m0 = tile_m * F::BM, n0 = tile_n * F::BN;
  const int iters = (Kp / F::BK) * npair;

  if(threadIdx.x == 0) {
    for(int s = 0; s < F::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    fence_mbar_init();
  }
  if(warp == 1) {
    umma::tmem_alloc(tmem_slot, F::TMEM_COLS);
    umma::tmem_relinquish();
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if(warp == 0) {
    // ------------------------------------------------------------ producer
    if(lane == 0) {
      for(int p = 0; p < npair; ++p)
        for(int t = 0; t < F::terms; ++t) {
          tma_prefetch_desc(&maps.p[p].l[t]);
          tma_prefetch_desc(&maps.p[p].r[t]);
        }
      int issued = 0;
      for(int it = 0; it < iters; ++it) {
        const int s = it % F::STAGES;
        if(it >= F::STAGES && !mbar_wait(&empty[s], ((it / F::STAGES) - 1) & 1, err, kDevErrEmptyWait)) break;
        const ProductMaps& pm = maps.p[it % npair];
        const int k0 = (it / npair) * F::BK;
        char* st = smem + s * F::STAGE;
        mbar_arrive_expect_tx(&full[s], F::STAGE);
#pragma unroll
        for(int t = 0; t < F::terms; ++t) {
          tma_load_2d(st + t * F::A_TILE, &pm.l[t], &full[s], k0, m0);
          tma_load_2d(st + F::terms * F::A_TILE + t * F::B_TILE, &pm.r[t], &full[s], k0, n0);
        }
        ++issued;
      }
      for(int it = max(0, issued - F::STAGES); it < issued; ++it)
        if(!mbar_wait(&full[it % F::STAGES], (it / F::STAGES) & 1, err, kDevErrDrainWait)) break;
    }
  } else if(warp == 1) {
    // ------------------------------------------------------------ MMA issue
    if(lane == 0) {
      for(int it = 0; it < iters; ++it) {
        const int s = it % F::STAGES;
        if(!mbar_wait(&full[s], (it / F::STAGES) & 1, err, kDevErrFullWait)) break;
        umma::fence_after_sync();
        const uint32_t a_base = smem_u32(smem + s * F::STAGE);
        const uint32_t b_base = a_base + F::terms * F::A_TILE;
#pragma unroll
        for(int k = 0; k < F::BK / F::KMMA; ++k) {
          const uint32_t off = k * 32;  // 32 bytes of K per MMA
#pragma unroll
          for(int p = 0; p < F::nprod; ++p) {
            const uint64_t da = umma::desc_k_sw128(a_base + prod_a(p) * F::A_TILE + off);
            const uint64_t db = umma::desc_k_sw128(b_base + prod_b(p) * F::B_TILE + off);
            const uint32_t acc = (it > 0 || k > 0 || p > 0) ? 1u : 0u;
            if constexpr(F::elem == Elem::BF16)
              umma::mma_f16(tmem, da, db, F::IDESC, acc);
            else
              umma::mma_tf32(tmem, da, db, F::IDESC, acc);
          }
        }
        umma::commit(&empty[s]);  // stage s is free once these MMAs have read it
      }
      umma::commit(accum);  // accumulator complete (after an error: all issued MMAs drained)
    }
  } else if(warp >= 4) {
    // ------------------------------------------------------------- epilogue
    const int q = warp & 3;
    const bool ok = mbar_wait(accum, 0, err, kDevErrMmaWait);
    umma::fence_after_sync();
    if(ok) {
      const int m = m0 + 32 * q + lane;
      float* crow = C + int64_t(m) * ldc;
      const bool vec = ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
#pragma unroll 1
      for(int c = 0; c < F::BN / 32; ++c) {
        uint32_t r[32];
        umma::tmem_ld_32x32b_x32(tmem + (uint32_t(32 * q) << 16) + uint32_t(32 * c), r);
        umma::tmem_ld_wait();
        const int n = n0 + 32 * c;
        if(m >= M || n >= N) continue;
        if(vec && n + 32 <= N) {
#pragma unroll
          for(int j = 0; j < 32; j += 4) {
            float4 o = make_float4(alpha * __uint_as_float(r[j]), alpha * __uint_as_float(r[j + 1]),
                alpha * __uint_as_float(r[j + 2]), alpha * __uint_as_float(r[j + 3]));
            if(beta != 0.f) {
              const float4 cv = *reinterpret_cast<const float4*>(crow + n + j);
              o.x = fmaf(beta, cv.x, o.x);
              o.y = fmaf(beta, cv.y, o.y);
              o.z = fmaf(beta, cv.z, o.z);
              o.w = fmaf(beta, cv.w, o.w);
            }
            *reinterpret_cast<float4*>(crow + n + j) = o;
          }
        } else {
#pragma unroll
          for(int j = 0; j < 32; ++j) {
            if(n + j < N) {
              const float v = alpha * __uint_as_float(r[j]);
              crow[n + j] = (beta != 0.f) ? fmaf(beta, crow[n + j], v) : v;
            }
          }
        }
      }
    }
  }

  umma::fence_before_sync();
  __syncthreads();
  if(warp == 1) {
    umma::fence_after_sync();
    if(lane == 0) mbar_wait(accum, 0, err, kDevErrDrainWait);  // no MMA may still write TMEM
    __syncwarp();
    umma::tmem_dealloc(tmem, F::TMEM_COLS);
  }
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Panels {
  char* base;     // term 0
  size_t stride;  // bytes between terms
};

template <class F>
gbpoly_status launch_split(gbpoly_ctx* ctx, const float* X, int64_t ld, bool k_major, int64_t rows, int64_t K,
    int64_t Kp, Panels out) {
  using T = typename Term<F::elem>::T;
  dim3 grid(static_cast<unsigned>(Kp / 64), static_cast<unsigned>((rows + 63) / 64));
  ProfileScope prof(ctx, "split_terms");
  split_kernel<F::elem, F::terms><<<grid, 256, 0, ctx->stream>>>(X, ld, k_major ? 1 : 0, int(rows), int(K), int(Kp),
      reinterpret_cast<T*>(out.base), int64_t(out.stride / sizeof(T)));
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

template <class F>
gbpoly_status make_product_maps(gbpoly_ctx* ctx, ProductMaps& pm, Panels left, int64_t left_rows, Panels right,
    int64_t right_rows, int64_t Kp) {
  const auto dt = F::elem == Elem::BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  const auto sw = CU_TENSOR_MAP_SWIZZLE_128B;
  gbpoly_status st;
  for(int t = 0; t < F::terms; ++t) {
    if((st = make_tmap_2d(ctx, &pm.l[t], dt, F::esz, left.base + t * left.stride, left_rows, Kp, Kp, F::BM, F::BK,
            sw)) != GBPOLY_OK)
      return st;
    if((st = make_tmap_2d(ctx, &pm.r[t], dt, F::esz, right.base + t * right.stride, right_rows, Kp, Kp, F::BN, F::BK,
            sw)) != GBPOLY_OK)
      return st;
  }
  return GBPOLY_OK;
}

template <class F>
gbpoly_status run_form(gbpoly_ctx* ctx, const GemmF32Args& a, const char* kernel_name) {
  if(a.M == 0 || a.N == 0) return GBPOLY_OK;
  if(a.M >= (1ll << 31) || a.N >= (1ll << 31) || a.K >= (1ll << 30))
    return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large for the tensor-core kernels");
  const int64_t Kp = align_up(size_t(std::max<int64_t>(a.K, 1)), 64);
  // syrk: both operands are the rows of A; split once
  const bool same = !a.dual && a.A == a.B && a.op_a == GBPOLY_OP_N && a.op_b == GBPOLY_OP_T && a.lda == a.ldb &&
                    a.M == a.N;
  const size_t a_stride = align_up(size_t(a.M) * Kp * F::esz, 1024);
  const size_t b_stride = align_up(size_t(a.N) * Kp * F::esz, 1024);
  const size_t a_bytes = F::terms * a_stride, b_bytes = same ? 0 : F::terms * b_stride;
  gbpoly_status st = ensure_workspace(ctx, a_bytes + b_bytes);
  if(st != GBPOLY_OK) return st;
  char* ws = static_cast<char*>(ctx->ws.ptr);
  Panels pa{ws, a_stride};
  Panels pb = same ? pa : Panels{ws + a_bytes, b_stride};
  if(a.K > 0) {
    if((st = launch_split<F>(ctx, a.A, a.lda, a.op_a == GBPOLY_OP_N, a.M, a.K, Kp, pa)) != GBPOLY_OK) return st;
    if(!same && (st = launch_split<F>(ctx, a.B, a.ldb, a.op_b == GBPOLY_OP_T, a.N, a.K, Kp, pb)) != GBPOLY_OK)
      return st;
  } else {
    GBPOLY_CUDA_TRY(cudaMemsetAsync(ws, 0, a_bytes + b_bytes, ctx->stream));
  }

  GemmMaps maps;
  int npair = 1;
  if((st = make_product_maps<F>(ctx, maps.p[0], pa, a.M, pb, a.N, Kp)) != GBPOLY_OK) return st;
  if(a.dual) {  // syr2k: second pairing B_i . A_j^T
    npair = 2;
    if((st = make_product_maps<F>(ctx, maps.p[1], pb, a.M, pa, a.N, Kp)) != GBPOLY_OK) return st;
  } else {
    maps.p[1] = maps.p[0];
  }

  static unsigned attr_set = 0;
  if(ctx->device < 32 && !(attr_set & (1u << ctx->device))) {
    GBPOLY_CUDA_TRY(cudaFuncSetAttribute(split_gemm_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, F::SMEM));
    attr_set |= 1u << ctx->device;
  }
  const int64_t tiles = ((a.M + F::BM - 1) / F::BM) * ((a.N + F::BN - 1) / F::BN);
  ProfileScope prof(ctx, kernel_name);
  split_gemm_kernel<F><<<static_cast<unsigned>(tiles), 256, F::SMEM, ctx->stream>>>(maps, npair, int(a.M), int(a.N),
      int(Kp), a.alpha, a.beta, a.C, a.ldc, ctx->err_dev);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

}  // namespace

gbpoly_status launch_gemm_tensor(gbpoly_ctx* ctx, gbpoly_precision prec, const GemmF32Args& a) {
  switch(prec) {
  case GBPOLY_PREC_TF32: return run_form<FormTF32>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_BF16X3: return run_form<FormBF16x3>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_TF32X3: return run_form<FormTF32x3>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_BF16X6: return run_form<FormBF16x6>(ctx, a, "bf16x6_gemm");
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision form not available");
  }
}

}  // namespace gbpoly
