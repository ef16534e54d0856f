// Plain FP32 SIMT contraction kernels for sm_103a: the drop-in form of the
// PolyBench kernels polybench/gemm.cpp:82-91, 2mm.cpp:99-122, 3mm.cpp:120-157,
// syrk.cpp:74-83 and syr2k.cpp:78-87.
//
// The reference launches one work-item per C element that walks the whole k
// range through global memory.  Here one CTA owns a 128x128 tile of C:
//   * one producer warp streams BK=32 slices of the A and B panels into a
//     ring of shared-memory stages with 2-D TMA (cp.async.bulk.tensor),
//     each stage guarded by a full/empty mbarrier pair;
//   * eight consumer warps (256 threads) each keep an 8x8 block of C in
//     registers and run FFMA over 128-bit shared-memory loads;
//   * the epilogue applies C = alpha*acc + beta*C with bounds checks.
// syr2k's two products (A_i.B_j + B_i.A_j) stream four tiles per stage into
// the same accumulator.  Symmetric updates (syrk, syr2k, X^T.X) compute only
// the tiles on and below the diagonal; a tile below it also stores its
// transpose (with its own beta * C term), so the full square is written.  Operands whose base or leading dimension is not
// 16-byte aligned (TMA's rule) take a simple tiled kernel without TMA.
#include "gbpoly_internal.cuh"
#include "tiled_gemm.cuh"

namespace gbpoly {
namespace {

constexpr int kBM = 128, kBN = 128, kBK = 32;
constexpr int kConsumers = 256;            // 8 consumer warps
constexpr int kThreads = kConsumers + 32;  // + 1 producer warp
constexpr int kTileBytes = kBM * kBK * 4;  // 16 KB, same for every tile shape used

// Byte offset of float4 chunk `chunk` (0..7) of row `row` in a [rows][32]
// fp32 tile written by TMA with 128-byte swizzle (chunk index XOR row%8).
__device__ __forceinline__ uint32_t swz128(int row, int chunk) {
  return static_cast<uint32_t>(row * 128 + ((chunk ^ (row & 7)) << 4));
}

// Operand tile layouts in shared memory:
//  K-major (k innermost, e.g. A as stored, or B^T as stored):
//     [128 rows][32 k], 128-byte swizzled.
//  MN-major (row/col innermost, e.g. B as stored for C = A.B):
//     [32 k][128], unswizzled 512-byte rows.
//
// Register fragment: v[i][kk] for the 8 rows (or columns) this thread owns
// and the 4 k values of one k-step.
//  MN-major: owned indices 4t..4t+3 and 64+4t..64+4t+3 (vector loads along the row).
//  K-major:  owned indices t+16i (rows t, t+16, ...), so that the 8 lanes of a
//            quarter warp hit 8 distinct swizzle phases (conflict-free).
template <bool KMAJ>
__device__ __forceinline__ int owned_index(int t, int i) {
  if constexpr(KMAJ)
    return t + 16 * i;
  else
    return (i < 4) ? (4 * t + i) : (64 + 4 * t + (i - 4));
}

template <bool KMAJ>
__device__ __forceinline__ void load_frag(const char* tile, int t, int kstep, float (&v)[8][4]) {
  if constexpr(KMAJ) {
#pragma unroll
    for(int i = 0; i < 8; ++i) {
      const int row = t + 16 * i;
      const float4 x = *reinterpret_cast<const float4*>(tile + swz128(row, kstep));
      v[i][0] = x.x;
      v[i][1] = x.y;
      v[i][2] = x.z;
      v[i][3] = x.w;
    }
  } else {
#pragma unroll
    for(int kk = 0; kk < 4; ++kk) {
      const char* rowp = tile + (kstep * 4 + kk) * 512;
      const float4 lo = *reinterpret_cast<const float4*>(rowp + 16 * t);
      const float4 hi = *reinterpret_cast<const float4*>(rowp + 256 + 16 * t);
      v[0][kk] = lo.x;
      v[1][kk] = lo.y;
      v[2][kk] = lo.z;
      v[3][kk] = lo.w;
      v[4][kk] = hi.x;
      v[5][kk] = hi.y;
      v[6][kk] = hi.z;
      v[7][kk] = hi.w;
    }
  }
}

template <bool A_KMAJ, bool B_KMAJ>
__device__ __forceinline__ void mma_tile(const char* ta, const char* tb, int tm, int tn, float (&acc)[8][8]) {
#pragma unroll 1
  for(int ks = 0; ks < kBK / 4; ++ks) {
    float a[8][4], b[8][4];
    load_frag<A_KMAJ>(ta, tm, ks, a);
    load_frag<B_KMAJ>(tb, tn, ks, b);
#pragma unroll
    for(int kk = 0; kk < 4; ++kk)
#pragma unroll
      for(int i = 0; i < 8; ++i)
#pragma unroll
        for(int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i][kk], b[j][kk], acc[i][j]);
  }
}

// Tile rasterisation: groups of 8 tile-rows walk the tile-columns together so
// that concurrently resident CTAs share A and B panels in L2.
__device__ __forceinline__ void tile_coords(int id, int tiles_m, int tiles_n, int& tile_m, int& tile_n) {
  constexpr int G = 8;
  const int per_group = G * tiles_n;
  const int group = id / per_group;
  const int first = group * G;
  const int gsz = min(tiles_m - first, G);
  const int r = id - group * per_group;
  tile_m = first + r % gsz;
  tile_n = r / gsz;
}

// Row-major walk of the lower triangle of tiles: t = tm (tm + 1) / 2 + tn, tn <= tm.
__device__ __forceinline__ void lower_coords(int t, int& tile_m, int& tile_n) {
  int tm = int((sqrtf(8.f * float(t) + 1.f) - 1.f) * 0.5f);
  while(tm * (tm + 1) / 2 > t) --tm;
  while((tm + 1) * (tm + 2) / 2 <= t) ++tm;
  tile_m = tm;
  tile_n = t - tm * (tm + 1) / 2;
}

// A_KMAJ: op(A) rows are contiguous in k (op_a == N).  B_KMAJ: op(B) columns
// are contiguous in k (op_b == T).  DUAL: syr2k, tiles A_i, B_j, B_i, A_j.
template <bool A_KMAJ, bool B_KMAJ, bool DUAL, int STAGES>
__global__ void __launch_bounds__(kThreads, 1) sgemm_tma_kernel(const __grid_constant__ CUtensorMap tmA,
    const __grid_constant__ CUtensorMap tmB, int M, int N, int K, float alpha, float beta, float* __restrict__ C,
    int64_t ldc, int lower, int kt_per_split, float* __restrict__ part, int* err) {
  constexpr int kTilesPerStage = DUAL ? 4 : 2;
  constexpr int kStageBytes = kTilesPerStage * kTileBytes;
  extern __shared__ __align__(1024) char smem_raw[];
  // 1024-byte aligned (128-byte swizzle atoms); offset arithmetic keeps the pointer in the shared window
  char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * kStageBytes);
  uint64_t* empty = full + STAGES;

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int tiles_m = (M + kBM - 1) / kBM, tiles_n = (N + kBN - 1) / kBN;
  int tile_m, tile_n;
  if(lower)
    lower_coords(blockIdx.x, tile_m, tile_n);
  else
    tile_coords(blockIdx.x, tiles_m, tiles_n, tile_m, tile_n);
  const int m0 = tile_m * kBM, n0 = tile_n * kBN;
  const bool mirror = lower && tile_m != tile_n;
  // split K (gridDim.y > 1): this CTA covers k tiles [kt0, kt0 + nkt) and
  // writes alpha * its partial product to its slice of `part` (M x N, ld N);
  // a reduction kernel adds the slices and beta * C
  const int ktiles = (K + kBK - 1) / kBK;
  const int kt0 = int(blockIdx.y) * kt_per_split;
  const int nkt = max(0, min(ktiles, kt0 + kt_per_split) - kt0);
  if(gridDim.y > 1) {
    C = part + int64_t(blockIdx.y) * int64_t(M) * N;
    ldc = N;
    beta = 0.f;
  }

  if(tid == 0) {
#pragma unroll
    for(int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumers / 32);
    }
    fence_mbar_init();
  }
  __syncthreads();

  if(warp == kConsumers / 32) {
    // ------------------------------------------------------------ producer
    if(lane == 0) {
      tma_prefetch_desc(&tmA);
      tma_prefetch_desc(&tmB);
      int issued = 0;
      for(int i = 0; i < nkt; ++i) {
        const int s = i % STAGES;
        if(i >= STAGES && !mbar_wait(&empty[s], ((i / STAGES) - 1) & 1, err, kDevErrEmptyWait)) break;
        char* st = smem + s * kStageBytes;
        mbar_arrive_expect_tx(&full[s], kStageBytes);
        const int k0 = (kt0 + i) * kBK;
        if constexpr(DUAL) {
          tma_load_2d(st + 0 * kTileBytes, &tmA, &full[s], k0, m0);  // A rows of the C tile
          tma_load_2d(st + 1 * kTileBytes, &tmB, &full[s], k0, n0);  // B rows of the C tile columns
          tma_load_2d(st + 2 * kTileBytes, &tmB, &full[s], k0, m0);
          tma_load_2d(st + 3 * kTileBytes, &tmA, &full[s], k0, n0);
        } else {
          if constexpr(A_KMAJ)
            tma_load_2d(st, &tmA, &full[s], k0, m0);
          else
            tma_load_2d(st, &tmA, &full[s], m0, k0);
          if constexpr(B_KMAJ)
            tma_load_2d(st + kTileBytes, &tmB, &full[s], k0, n0);
          else
            tma_load_2d(st + kTileBytes, &tmB, &full[s], n0, k0);
        }
        ++issued;
      }
      // Drain: do not leave the CTA while copies into its shared memory are in flight.
      for(int kt = max(0, issued - STAGES); kt < issued; ++kt) {
        if(!mbar_wait(&full[kt % STAGES], (kt / STAGES) & 1, err, kDevErrDrainWait)) break;
      }
    }
    return;
  }

  // -------------------------------------------------------------- consumers
  const int tm = warp * 2 + (lane >> 4);  // 0..15
  const int tn = lane & 15;               // 0..15
  float acc[8][8];
#pragma unroll
  for(int i = 0; i < 8; ++i)
#pragma unroll
    for(int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  bool ok = true;
  for(int kt = 0; kt < nkt; ++kt) {
    if(kt == max(0, nkt - 4) && beta != 0.f) {
      // C of the tile (and of its mirror) into L2 a few k tiles before the
      // epilogue reads it: 512 lines of 128 bytes, two per consumer thread
#pragma unroll
      for(int e = 0; e < 2; ++e) {
        const int line = tid + kConsumers * e, r = line >> 2, c = 32 * (line & 3);
        if(m0 + r < M && n0 + c < N) prefetch_l2(C + int64_t(m0 + r) * ldc + n0 + c);
        if(mirror && n0 + r < N && m0 + c < M) prefetch_l2(C + int64_t(n0 + r) * ldc + m0 + c);
      }
    }
    const int s = kt % STAGES;
    if(!mbar_wait(&full[s], (kt / STAGES) & 1, err, kDevErrFullWait)) {
      ok = false;
      break;
    }
    const char* st = smem + s * kStageBytes;
    if constexpr(DUAL) {
      mma_tile<true, true>(st + 0 * kTileBytes, st + 1 * kTileBytes, tm, tn, acc);
      mma_tile<true, true>(st + 2 * kTileBytes, st + 3 * kTileBytes, tm, tn, acc);
    } else {
      mma_tile<A_KMAJ, B_KMAJ>(st, st + kTileBytes, tm, tn, acc);
    }
    __syncwarp();
    if(lane == 0) mbar_arrive(&empty[s]);
  }
  if(!ok) return;

  // --------------------------------------------------------------- epilogue
  // C = alpha * acc + beta * C, four rows (then, below the diagonal of a
  // symmetric product, four transposed rows) at a time: the 32 C values of a
  // group are loaded before the group's first store.  A load cannot move above
  // a store that may alias it, so interleaving them per element would
  // serialise one memory round trip per element.
  constexpr bool kVecCols = !B_KMAJ && !DUAL;
  const bool vec_ok = kVecCols && ((ldc & 3) == 0) && ((reinterpret_cast<uintptr_t>(C) & 15) == 0);
  int rm[8], cn[8];  // owned rows (m) and columns (n)
#pragma unroll
  for(int i = 0; i < 8; ++i) rm[i] = m0 + owned_index<A_KMAJ || DUAL>(tm, i);
#pragma unroll
  for(int j = 0; j < 8; ++j) cn[j] = n0 + owned_index<B_KMAJ || DUAL>(tn, j);
  const bool read_c = beta != 0.f;
#pragma unroll
  for(int g = 0; g < 8; g += 4) {
    float cv[4][8];
#pragma unroll
    for(int r = 0; r < 4; ++r) {
      const int i = g + r;
      const float* crow = C + static_cast<int64_t>(rm[i]) * ldc;
#pragma unroll
      for(int h = 0; h < 2; ++h) {
        if(read_c && vec_ok && rm[i] < M && cn[4 * h] + 3 < N) {
          const float4 c = *reinterpret_cast<const float4*>(crow + cn[4 * h]);
          cv[r][4 * h + 0] = c.x, cv[r][4 * h + 1] = c.y, cv[r][4 * h + 2] = c.z, cv[r][4 * h + 3] = c.w;
        } else {
#pragma unroll
          for(int q = 0; q < 4; ++q)
            cv[r][4 * h + q] = (read_c && rm[i] < M && cn[4 * h + q] < N) ? crow[cn[4 * h + q]] : 0.f;
        }
      }
    }
#pragma unroll
    for(int r = 0; r < 4; ++r) {
      const int i = g + r;
      if(rm[i] >= M) continue;
      float* crow = C + static_cast<int64_t>(rm[i]) * ldc;
#pragma unroll
      for(int h = 0; h < 2; ++h) {
        float o[4];
#pragma unroll
        for(int q = 0; q < 4; ++q) o[q] = fmaf(beta, cv[r][4 * h + q], alpha * acc[i][4 * h + q]);
        if(vec_ok && cn[4 * h] + 3 < N) {
          *reinterpret_cast<float4*>(crow + cn[4 * h]) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
#pragma unroll
          for(int q = 0; q < 4; ++q)
            if(cn[4 * h + q] < N) crow[cn[4 * h + q]] = o[q];
        }
      }
    }
  }
  if(mirror) {  // C[n][m] from the product element (m, n): the tile's transpose, strictly above the diagonal
#pragma unroll
    for(int g = 0; g < 8; g += 4) {
      float mv[4][8];
#pragma unroll
      for(int r = 0; r < 4; ++r)
#pragma unroll
        for(int i = 0; i < 8; ++i)
          mv[r][i] = (read_c && cn[g + r] < N && rm[i] < M) ? C[static_cast<int64_t>(cn[g + r]) * ldc + rm[i]] : 0.f;
#pragma unroll
      for(int r = 0; r < 4; ++r) {
        const int j = g + r;
        if(cn[j] >= N) continue;
        float* crow = C + static_cast<int64_t>(cn[j]) * ldc;
#pragma unroll
        for(int i = 0; i < 8; ++i)
          if(rm[i] < M) crow[rm[i]] = fmaf(beta, mv[r][i], alpha * acc[i][j]);
      }
    }
  }
}

// C = sum over the splits of part[s] (already scaled by alpha) + beta C, the
// splits added in index order.
__global__ void split_k_reduce_kernel(const float* __restrict__ part, int splits, int M, int N, float beta, float* C,
    int64_t ldc) {
  const int64_t total = int64_t(M) * N;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for(int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += stride) {
    const int64_t m = e / N, n = e - m * N;
    float s = 0.f;
    for(int k = 0; k < splits; ++k) s += part[int64_t(k) * total + e];
    float* c = C + m * ldc + n;
    *c = beta != 0.f ? fmaf(beta, *c, s) : s;
  }
}

// K split for grids too small to fill the device: about one CTA per SM, at
// least 4 k tiles (128 of K) per split, at most 8 splits.
int split_k_count(int sm_count, int64_t tiles, int64_t ktiles) {
  if(tiles <= 0 || tiles * 2 > sm_count || ktiles < 8) return 1;
  int64_t s = std::min<int64_t>(std::min<int64_t>(sm_count / tiles, ktiles / 4), 8);
  if(s <= 1) return 1;
  const int64_t per = (ktiles + s - 1) / s;
  return int((ktiles + per - 1) / per);  // every split non-empty
}

template <bool A_KMAJ, bool B_KMAJ, bool DUAL, int STAGES>
gbpoly_status launch_tma(gbpoly_ctx* ctx, const GemmF32Args& a, const CUtensorMap& ta, const CUtensorMap& tb,
    bool lower) {
  constexpr int kStageBytes = (DUAL ? 4 : 2) * kTileBytes;
  constexpr int kSmem = STAGES * kStageBytes + 1024 + 2 * STAGES * 8;
  auto kern = sgemm_tma_kernel<A_KMAJ, B_KMAJ, DUAL, STAGES>;
  static ContextMark attr_set;  // the attribute is set once per device context
  if(!attr_set.valid(ctx->device)) {
    GBPOLY_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem));
    attr_set.set(ctx->device);
  }
  int64_t tiles = ((a.M + kBM - 1) / kBM) * ((a.N + kBN - 1) / kBN);
  if(lower) {
    const int64_t t = (a.M + kBM - 1) / kBM;
    tiles = t * (t + 1) / 2;
  }
  // the split depends on the full square's tile count, so a symmetric product
  // splits K exactly like the same product computed in full (same bits)
  const int64_t ktiles = (a.K + kBK - 1) / kBK;
  int splits = a.ksplit > 0 ? int(std::min<int64_t>(a.ksplit, std::max<int64_t>(ktiles, 1)))
                            : split_k_count(ctx->sm_count, ((a.M + kBM - 1) / kBM) * ((a.N + kBN - 1) / kBN), ktiles);
  const int kt_per_split = int((ktiles + splits - 1) / splits);
  splits = int((ktiles + kt_per_split - 1) / kt_per_split);  // every split non-empty
  if(splits < 1) splits = 1;
  float* part = nullptr;
  if(splits > 1) {
    gbpoly_status st = ensure_workspace(ctx, size_t(splits) * size_t(a.M) * size_t(a.N) * sizeof(float));
    if(st != GBPOLY_OK) return st;
    part = static_cast<float*>(ctx->ws.ptr);
  }
  {
    ProfileScope prof(ctx, DUAL ? "sgemm_simt_dual" : "sgemm_simt");
    kern<<<dim3(static_cast<unsigned>(tiles), static_cast<unsigned>(splits)), kThreads, kSmem, ctx->stream>>>(ta, tb,
        static_cast<int>(a.M), static_cast<int>(a.N), static_cast<int>(a.K), a.alpha, a.beta, a.C, a.ldc,
        lower ? 1 : 0, kt_per_split, part, ctx->err_dev);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  if(splits > 1) {
    ProfileScope prof(ctx, "split_k_reduce");
    const int64_t total = a.M * a.N;
    const unsigned blocks = unsigned(std::min<int64_t>((total + 255) / 256, 8ll * ctx->sm_count));
    split_k_reduce_kernel<<<blocks, 256, 0, ctx->stream>>>(part, splits, int(a.M), int(a.N), a.beta, a.C, a.ldc);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  return GBPOLY_OK;
}

}  // namespace

// Workspace bytes of the K split of an FP32 contraction, for a device of at
// most `sm_count` SMs (more SMs never need less).
int fp32_split_k_count(int sm_count, int64_t M, int64_t N, int64_t K) {
  return split_k_count(sm_count, ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN), (K + kBK - 1) / kBK);
}

size_t fp32_split_k_bytes(int sm_count, int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + kBM - 1) / kBM) * ((N + kBN - 1) / kBN);
  const int s = split_k_count(sm_count, tiles, (K + kBK - 1) / kBK);
  return s > 1 ? size_t(s) * size_t(M) * size_t(N) * sizeof(float) : 0;
}

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace

gbpoly_status launch_gemm_f32_simt(gbpoly_ctx* ctx, const GemmF32Args& a) {
  if(a.M == 0 || a.N == 0) return GBPOLY_OK;
  const bool a_kmaj = a.op_a == GBPOLY_OP_N;
  const bool b_kmaj = a.op_b == GBPOLY_OP_T;
  bool tma_ok = aligned16(a.A) && aligned16(a.B) && (a.lda % 4 == 0) && (a.ldb % 4 == 0) && a.K > 0 &&
                a.M < (1ll << 31) && a.N < (1ll << 31) && a.K < (1ll << 31);
  if(a.dual) tma_ok = tma_ok && a_kmaj && b_kmaj && a.A2 == a.B && a.B2 == a.A;

  if(!tma_ok) {
    TiledOperand<float> oa = a_kmaj ? TiledOperand<float>{a.A, a.lda, 1} : TiledOperand<float>{a.A, 1, a.lda};
    TiledOperand<float> ob = b_kmaj ? TiledOperand<float>{a.B, a.ldb, 1} : TiledOperand<float>{a.B, 1, a.ldb};
    TiledOperand<float> oa2{a.A2, a.lda2, 1}, ob2{a.B2, a.ldb2, 1};
    return launch_tiled_gemm<float>(ctx, a.M, a.N, a.K, a.alpha, oa, ob, a.dual, oa2, ob2, a.beta, a.C, a.ldc,
        a.M == a.N && (a.dual || symmetric_operand(a)));
  }

  CUtensorMap ta, tb;
  const auto dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  gbpoly_status st;
  // op(A) is M x K.  Stored as M x K (K-major) for op N, K x M for op T.
  if(a_kmaj)
    st = make_tmap_2d(ctx, &ta, dt, 4, a.A, a.M, a.K, a.lda, kBM, kBK, CU_TENSOR_MAP_SWIZZLE_128B);
  else
    st = make_tmap_2d(ctx, &ta, dt, 4, a.A, a.K, a.M, a.lda, kBK, kBM, CU_TENSOR_MAP_SWIZZLE_NONE);
  if(st != GBPOLY_OK) return st;
  // op(B) is K x N.  Stored as K x N for op N, N x K (K-major) for op T.
  if(b_kmaj)
    st = make_tmap_2d(ctx, &tb, dt, 4, a.B, a.N, a.K, a.ldb, kBN, kBK, CU_TENSOR_MAP_SWIZZLE_128B);
  else
    st = make_tmap_2d(ctx, &tb, dt, 4, a.B, a.K, a.N, a.ldb, kBK, kBN, CU_TENSOR_MAP_SWIZZLE_NONE);
  if(st != GBPOLY_OK) return st;

  // Symmetric product (op(A) == op(B)^T as stored, or syr2k): lower triangle of tiles only.
  const bool lower = a.M == a.N && (a.dual || symmetric_operand(a));
  if(a.dual) return launch_tma<true, true, true, 3>(ctx, a, ta, tb, lower);
  if(a_kmaj && b_kmaj) return launch_tma<true, true, false, 4>(ctx, a, ta, tb, lower);
  if(a_kmaj && !b_kmaj) return launch_tma<true, false, false, 4>(ctx, a, ta, tb, lower);
  if(!a_kmaj && b_kmaj) return launch_tma<false, true, false, 4>(ctx, a, ta, tb, lower);
  return launch_tma<false, false, false, 4>(ctx, a, ta, tb, lower);
}

}  // namespace gbpoly
