// Matrix-vector products of the PolyBench BLAS-2 benchmarks (atax, bicg,
// mvt, gesummv), HBM-bound: every kernel reads each matrix element once.
//
// The reference runs one work-item per output element: row dots walk a row
// per work-item (uncoalesced across the work-group), column sums walk a
// column (polybench/atax.cpp:73-97, bicg.cpp:77-100, mvt.cpp:75-98,
// gesummv.cpp:84-98).  Here one pass over the matrix serves up to two row
// dots (y = A x, or A x and B x for gesummv) and one column sum (A^T v):
//   * a CTA of 256 threads owns a 1024-column tile (4 adjacent columns per
//     thread, 128-bit loads) and a group of rows; each row of the tile is one
//     coalesced 4 KB read, 16 rows in flight per thread (8 per matrix for two);
//   * row dots: a thread's 4 columns give one term per row; each group of 8
//     rows in flight is reduced across the warp at once (a halving transpose
//     exchange: 16 shuffles for 16 rows), the 8 warps in shared memory per
//     32-row block, into one partial per (column tile, row);
//   * column sums: 4 accumulators per thread over all rows of the group,
//     one partial per (row group, column);
//   * a final kernel (8 warps per 32 outputs) adds the partials in a fixed order and applies
//     y = beta * y + alpha * sum (gesummv: tmp += A x, y = alpha tmp + beta (y + B x)).
// Deterministic: the summation tree depends only on the shape and SM count.
#include "gbpoly_internal.cuh"

namespace gbpoly {
namespace {

constexpr int kThreads = 256;
constexpr int kTileCols = 4 * kThreads;  // 1024
constexpr int kRowBlock = 32;
// rows in flight per thread: 16 for one matrix, 8 each for two (gesummv)
template <bool TWO>
constexpr int rows_in_flight() {
  return TWO ? 8 : 16;
}

struct GemvArgs {
  const float* A;
  int64_t lda;
  const float* B;  // second matrix (gesummv), row dot 1 reads it with xr[1]
  int64_t ldb;
  int rows, cols;
  const float* xr[2];  // row-dot vectors (cols entries)
  const float* xc;     // column-sum weights (rows entries)
  float* row_part;     // [NR][col_tiles][rows]
  float* col_part;     // [row_groups][cols]
  int col_tiles, rows_per_group;
};

__device__ __forceinline__ float4 load4(const float* p, int c, int cols, bool vec) {
  if(vec) return *reinterpret_cast<const float4*>(p + c);
  float4 v;
  v.x = c < cols ? p[c] : 0.f;
  v.y = c + 1 < cols ? p[c + 1] : 0.f;
  v.z = c + 2 < cols ? p[c + 2] : 0.f;
  v.w = c + 3 < cols ? p[c + 3] : 0.f;
  return v;
}

__device__ __forceinline__ float dot4(float4 a, float4 x) {
  return fmaf(a.w, x.w, fmaf(a.z, x.z, fmaf(a.y, x.y, a.x * x.x)));
}

// Warp-wide sums of V (8 or 16) values per lane: halving exchanges (V/2 +
// ... + 1 shuffles) leave lane l with the sum of v[l % V] over its group of V
// lanes, butterfly steps add the 32 / V groups.  Every lane ends with the
// total of v[lane % V].
template <int V>
__device__ __forceinline__ float reduce_rows(float (&v)[V], int lane) {
#pragma unroll
  for(int s = V / 2; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
#pragma unroll
    for(int i = 0; i < s; ++i) {
      const float send = upper ? v[i] : v[i + s];
      const float keep = upper ? v[i + s] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, s);
    }
  }
  float r = v[0];
#pragma unroll
  for(int s = V; s < 32; s <<= 1) r += __shfl_xor_sync(0xffffffffu, r, s);
  return r;
}

// NR row dots (0..2), NC: one column sum, TWO: row dot 1 reads B.
// VEC: 16-byte aligned rows and columns a multiple of 4 (128-bit loads).
template <int NR, bool NC, bool TWO, bool VEC>
__global__ void __launch_bounds__(kThreads, 2) gemv_partial_kernel(const GemvArgs g) {
  __shared__ float red[NR > 0 ? NR : 1][kThreads / 32][kRowBlock];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile = blockIdx.x;
  const int c = tile * kTileCols + 4 * tid;
  const bool col_ok = c < g.cols;
  const int rg0 = blockIdx.y * g.rows_per_group;
  const int rg1 = min(g.rows, rg0 + g.rows_per_group);

  float4 xr[NR > 0 ? NR : 1];
#pragma unroll
  for(int t = 0; t < NR; ++t) xr[t] = col_ok ? load4(g.xr[t], c, g.cols, VEC) : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 colacc = make_float4(0.f, 0.f, 0.f, 0.f);

  constexpr int kInFlight = rows_in_flight<TWO>();
  for(int r0 = rg0; r0 < rg1; r0 += kRowBlock) {
    // a thread's 4 columns of a row give one term of that row's dot product;
    // each group of rows in flight is reduced across the warp at once
#pragma unroll 1
    for(int rr = 0; rr < kRowBlock; rr += kInFlight) {
      float4 a[kInFlight], b[TWO ? kInFlight : 1];
#pragma unroll
      for(int k = 0; k < kInFlight; ++k) {
        const int r = r0 + rr + k;
        const bool ok = col_ok && r < rg1;
        a[k] = ok ? load4(g.A + int64_t(r) * g.lda, c, g.cols, VEC) : make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr(TWO) b[k] = ok ? load4(g.B + int64_t(r) * g.ldb, c, g.cols, VEC) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for(int t = 0; t < NR; ++t) {
        float v[kInFlight];
#pragma unroll
        for(int k = 0; k < kInFlight; ++k) v[k] = dot4((TWO && t == 1) ? b[TWO ? k : 0] : a[k], xr[t]);
        const float rs = reduce_rows<kInFlight>(v, lane);
        if(lane < kInFlight) red[t][warp][rr + lane] = rs;
      }
      if constexpr(NC) {
#pragma unroll
        for(int k = 0; k < kInFlight; ++k) {
          const int r = r0 + rr + k;
          const float w = r < rg1 ? __ldg(g.xc + r) : 0.f;
          colacc.x = fmaf(a[k].x, w, colacc.x);
          colacc.y = fmaf(a[k].y, w, colacc.y);
          colacc.z = fmaf(a[k].z, w, colacc.z);
          colacc.w = fmaf(a[k].w, w, colacc.w);
        }
      }
    }
    if constexpr(NR > 0) {
      __syncthreads();
      if(warp < NR) {
        float s = 0.f;
#pragma unroll
        for(int w = 0; w < kThreads / 32; ++w) s += red[warp][w][lane];
        const int r = r0 + lane;
        if(r < rg1) g.row_part[(int64_t(warp) * g.col_tiles + tile) * g.rows + r] = s;
      }
      __syncthreads();
    }
  }
  if constexpr(NC) {
    float* out = g.col_part + int64_t(blockIdx.y) * g.cols;
    if(VEC && c + 3 < g.cols) {
      *reinterpret_cast<float4*>(out + c) = colacc;
    } else {
      if(c < g.cols) out[c] = colacc.x;
      if(c + 1 < g.cols) out[c + 1] = colacc.y;
      if(c + 2 < g.cols) out[c + 2] = colacc.z;
      if(c + 3 < g.cols) out[c + 3] = colacc.w;
    }
  }
}

struct Term {
  float alpha, beta;
  float* y;
};

// alpha * s + beta * y[i]; y is not read when beta == 0 (NaN in y does not propagate)
__device__ __forceinline__ float apply(const Term& t, float s, int i) {
  return t.beta == 0.f ? t.alpha * s : fmaf(t.alpha, s, t.beta * t.y[i]);
}

// Final pass, one CTA per 32 outputs: warp w adds the partials with index
// w, w + 8, ... of output (blockIdx.x * 32 + lane); the 8 warp sums are
// combined in shared memory in warp order.
//   row terms:   y_r[i] = beta y_r[i] + alpha sum over column tiles of row_part[t][.][i]
//   column term: y_c[j] = beta y_c[j] + alpha sum over row groups of col_part[.][j]
//   GESUMMV:     tmp += S0, y = alpha tmp + beta (y + S1) (row terms 0, 1)
template <int NR, bool NC, bool GESUMMV>
__global__ void __launch_bounds__(256) gemv_final_kernel(const float* __restrict__ row_part, int col_tiles, int rows,
    const float* __restrict__ col_part, int row_groups, int cols, Term r0, Term r1, Term cterm) {
  constexpr int kSums = (NR > 0 ? NR : 0) + (NC ? 1 : 0);
  __shared__ float red[kSums > 0 ? kSums : 1][8][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  if constexpr(NR > 0) {
#pragma unroll
    for(int t = 0; t < NR; ++t) {
      float s = 0.f;
      if(i < rows)
        for(int ct = warp; ct < col_tiles; ct += 8) s += row_part[(int64_t(t) * col_tiles + ct) * rows + i];
      red[t][warp][lane] = s;
    }
  }
  if constexpr(NC) {
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // four loads in flight
    if(i < cols) {
      int g = warp;
      for(; g + 24 < row_groups; g += 32) {
        s0 += col_part[int64_t(g) * cols + i];
        s1 += col_part[int64_t(g + 8) * cols + i];
        s2 += col_part[int64_t(g + 16) * cols + i];
        s3 += col_part[int64_t(g + 24) * cols + i];
      }
      for(; g < row_groups; g += 8) s0 += col_part[int64_t(g) * cols + i];
    }
    red[kSums - 1][warp][lane] = (s0 + s1) + (s2 + s3);
  }
  __syncthreads();
  if(warp != 0) return;
  float sum[kSums > 0 ? kSums : 1];
#pragma unroll
  for(int t = 0; t < kSums; ++t) {
    sum[t] = 0.f;
#pragma unroll
    for(int w = 0; w < 8; ++w) sum[t] += red[t][w][lane];
  }
  if(NR > 0 && i < rows) {
    if constexpr(GESUMMV) {
      const float tmp = r0.y[i] + sum[0];
      r0.y[i] = tmp;
      r1.y[i] = r1.beta == 0.f ? r1.alpha * tmp : fmaf(r1.alpha, tmp, r1.beta * (r1.y[i] + sum[NR > 1 ? 1 : 0]));
    } else {
      r0.y[i] = apply(r0, sum[0], i);
      if constexpr(NR > 1) r1.y[i] = apply(r1, sum[NR > 1 ? 1 : 0], i);
    }
  }
  if(NC && i < cols) cterm.y[i] = apply(cterm, sum[kSums - 1], i);
}

template <int NR, bool NC, bool TWO, bool GESUMMV>
gbpoly_status launch_gemv(gbpoly_ctx* ctx, GemvArgs g, Term r0, Term r1, Term ct, const char* name) {
  // An empty matrix runs only the final kernel, with empty sums: y = beta y,
  // and for gesummv tmp unchanged, y = alpha tmp + beta y.
  const int col_tiles = std::max(1, (g.cols + kTileCols - 1) / kTileCols);
  const int64_t want_groups = std::max<int64_t>(1, (4ll * std::max(ctx->sm_count, 1) + col_tiles - 1) / col_tiles);
  int rpg = int((int64_t(g.rows) + want_groups - 1) / want_groups);
  rpg = std::max(kRowBlock, (rpg + kRowBlock - 1) / kRowBlock * kRowBlock);
  const int row_groups = std::max(1, (g.rows + rpg - 1) / rpg);
  if(row_groups > 65535) return fail(GBPOLY_ERR_UNSUPPORTED, "too many rows");
  g.col_tiles = col_tiles;
  g.rows_per_group = rpg;
  const size_t row_floats = size_t(NR) * col_tiles * size_t(g.rows);
  const size_t col_floats = NC ? size_t(row_groups) * size_t(g.cols) : 0;
  const size_t row_bytes = (row_floats * 4 + 255) / 256 * 256;
  gbpoly_status st = ensure_scratch(ctx, ctx->stats, row_bytes + col_floats * 4 + 256, "matrix-vector scratch");
  if(st != GBPOLY_OK) return st;
  g.row_part = static_cast<float*>(ctx->stats.ptr);
  g.col_part = reinterpret_cast<float*>(static_cast<char*>(ctx->stats.ptr) + row_bytes);
  const bool vec = (g.cols % 4 == 0) && (g.lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.A) & 15) == 0) &&
                   (!TWO || ((g.ldb % 4 == 0) && ((reinterpret_cast<uintptr_t>(g.B) & 15) == 0))) &&
                   (NR < 1 || (reinterpret_cast<uintptr_t>(g.xr[0]) & 15) == 0) &&
                   (NR < 2 || (reinterpret_cast<uintptr_t>(g.xr[1]) & 15) == 0);
  if(g.rows > 0 && g.cols > 0) {
    ProfileScope prof(ctx, name);
    const dim3 grid{unsigned(col_tiles), unsigned(row_groups), 1u};
    if(vec)
      gemv_partial_kernel<NR, NC, TWO, true><<<grid, kThreads, 0, ctx->stream>>>(g);
    else
      gemv_partial_kernel<NR, NC, TWO, false><<<grid, kThreads, 0, ctx->stream>>>(g);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  const int n = std::max(g.rows, g.cols);
  if(n == 0) return GBPOLY_OK;
  ProfileScope prof(ctx, "gemv_final");
  gemv_final_kernel<NR, NC, GESUMMV><<<unsigned((n + 31) / 32), 256, 0, ctx->stream>>>(g.row_part,
      (g.rows > 0 && g.cols > 0) ? col_tiles : 0, g.rows, g.col_part, (g.rows > 0 && g.cols > 0) ? row_groups : 0,
      g.cols, r0, r1, ct);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

// atax in one kernel: tmp += A x, then y += A^T tmp, each row group's rows
// read from HBM once.  A persistent CTA walks row groups of kAtaxRows rows:
// phase 1 reads the group's rows over all column chunks and completes their
// row dots (so tmp of those rows is final), phase 2 reads the same rows again
// (just read: from L2) and adds A[r][c] tmp[r] into the thread's column
// accumulators, which stay in registers across the CTA's row groups and are
// written once as the CTA's partial row of col_part.  CHUNKS 1024-column
// chunks (cols <= CHUNKS * 1024, at most 8), 128-bit loads, one CTA per SM.
constexpr int kAtaxRows = 16;

template <int CHUNKS>
__global__ void __launch_bounds__(kThreads, 1) atax_kernel(const float* __restrict__ A, int64_t lda, int rows, int cols,
    const float* __restrict__ x, float* __restrict__ tmp, float* __restrict__ col_part, int groups) {
  __shared__ float red[kThreads / 32][kAtaxRows];
  __shared__ float tmp_s[kAtaxRows];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float4 xr[CHUNKS], colacc[CHUNKS];
#pragma unroll
  for(int ch = 0; ch < CHUNKS; ++ch) {
    const int c = ch * kTileCols + 4 * tid;
    xr[ch] = c < cols ? *reinterpret_cast<const float4*>(x + c) : make_float4(0.f, 0.f, 0.f, 0.f);
    colacc[ch] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for(int g = blockIdx.x; g < groups; g += gridDim.x) {
    const int r0 = g * kAtaxRows, nr = min(kAtaxRows, rows - r0);
    // phase 1: row dots of the group over all columns
    float acc[kAtaxRows];
#pragma unroll
    for(int k = 0; k < kAtaxRows; ++k) acc[k] = 0.f;
#pragma unroll
    for(int ch = 0; ch < CHUNKS; ++ch) {
      const int c = ch * kTileCols + 4 * tid;
      if(c < cols) {
        float4 a[kAtaxRows];
#pragma unroll
        for(int k = 0; k < kAtaxRows; ++k)
          a[k] = k < nr ? *reinterpret_cast<const float4*>(A + int64_t(r0 + k) * lda + c) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for(int k = 0; k < kAtaxRows; ++k) acc[k] += dot4(a[k], xr[ch]);
      }
    }
    const float rs = reduce_rows<kAtaxRows>(acc, lane);
    if(lane < kAtaxRows) red[warp][lane] = rs;
    __syncthreads();
    if(warp == 0 && lane < kAtaxRows) {
      float sum = 0.f;
#pragma unroll
      for(int w = 0; w < kThreads / 32; ++w) sum += red[w][lane];
      float t = 0.f;
      if(lane < nr) {
        t = tmp[r0 + lane] + sum;  // tmp += A x (atax.cpp:78-83)
        tmp[r0 + lane] = t;
      }
      tmp_s[lane] = t;
    }
    __syncthreads();
    // phase 2: the same rows again, y += A^T tmp (atax.cpp:91-96)
#pragma unroll
    for(int ch = 0; ch < CHUNKS; ++ch) {
      const int c = ch * kTileCols + 4 * tid;
      if(c < cols) {
        float4 a[kAtaxRows];
#pragma unroll
        for(int k = 0; k < kAtaxRows; ++k)
          a[k] = k < nr ? *reinterpret_cast<const float4*>(A + int64_t(r0 + k) * lda + c) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for(int k = 0; k < kAtaxRows; ++k) {
          const float w = tmp_s[k];
          colacc[ch].x = fmaf(a[k].x, w, colacc[ch].x);
          colacc[ch].y = fmaf(a[k].y, w, colacc[ch].y);
          colacc[ch].z = fmaf(a[k].z, w, colacc[ch].z);
          colacc[ch].w = fmaf(a[k].w, w, colacc[ch].w);
        }
      }
    }
    __syncthreads();  // red and tmp_s are rewritten by the next group
  }
#pragma unroll
  for(int ch = 0; ch < CHUNKS; ++ch) {
    const int c = ch * kTileCols + 4 * tid;
    if(c < cols) *reinterpret_cast<float4*>(col_part + int64_t(blockIdx.x) * cols + c) = colacc[ch];
  }
}

template <int CHUNKS>
gbpoly_status launch_atax(gbpoly_ctx* ctx, const float* A, int64_t lda, int rows, int cols, const float* x, float* tmp,
    float* y) {
  const int groups = (rows + kAtaxRows - 1) / kAtaxRows;
  const int grid = std::max(1, std::min(groups, std::max(ctx->sm_count, 1)));  // one CTA per SM
  gbpoly_status st = ensure_scratch(ctx, ctx->stats, size_t(grid) * size_t(cols) * 4 + 256, "matrix-vector scratch");
  if(st != GBPOLY_OK) return st;
  float* col_part = static_cast<float*>(ctx->stats.ptr);
  {
    ProfileScope prof(ctx, "atax");
    atax_kernel<CHUNKS><<<grid, kThreads, 0, ctx->stream>>>(A, lda, rows, cols, x, tmp, col_part, groups);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  ProfileScope prof(ctx, "gemv_final");
  gemv_final_kernel<0, true, false><<<unsigned((cols + 31) / 32), 256, 0, ctx->stream>>>(nullptr, 0, rows, col_part,
      grid, cols, Term{}, Term{}, Term{1.f, 1.f, y});
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

gbpoly_status check_common(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* A, int64_t lda) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  if(rows < 0 || cols < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  if(rows >= (1ll << 31) || cols >= (1ll << 31) - kTileCols) return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large");
  if(rows > 0 && cols > 0) {
    if(!A) return fail(GBPOLY_ERR_INVALID, "matrix: null pointer");
    if(lda < cols) return fail(GBPOLY_ERR_INVALID, "matrix: leading dimension smaller than columns");
  }
  return GBPOLY_OK;
}

}  // namespace
}  // namespace gbpoly

using namespace gbpoly;

extern "C" {

gbpoly_status gbpoly_gemv_pair_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* A, int64_t lda,
    const gbpoly_gemv_term* terms, int count) {
  gbpoly_status st = check_common(ctx, rows, cols, A, lda);
  if(st != GBPOLY_OK) return st;
  if(!terms || count < 1 || count > 2) return fail(GBPOLY_ERR_INVALID, "one or two terms");
  const gbpoly_gemv_term* rt[2] = {nullptr, nullptr};
  const gbpoly_gemv_term* cterm = nullptr;
  int nr = 0;
  for(int i = 0; i < count; ++i) {
    const gbpoly_gemv_term& t = terms[i];
    if(t.op != GBPOLY_OP_N && t.op != GBPOLY_OP_T) return fail(GBPOLY_ERR_INVALID, "bad term op");
    const int64_t xlen = t.op == GBPOLY_OP_N ? cols : rows, ylen = t.op == GBPOLY_OP_N ? rows : cols;
    if((xlen > 0 && !t.x) || (ylen > 0 && !t.y)) return fail(GBPOLY_ERR_INVALID, "term vector: null pointer");
    if(t.op == GBPOLY_OP_N) {
      rt[nr++] = &t;
    } else {
      if(cterm) return fail(GBPOLY_ERR_UNSUPPORTED, "at most one transposed term");
      cterm = &t;
    }
  }
  GemvArgs g{};
  g.A = A, g.lda = lda, g.rows = int(rows), g.cols = int(cols);
  Term r0{}, r1{}, ct{};
  if(nr > 0) g.xr[0] = rt[0]->x, r0 = Term{rt[0]->alpha, rt[0]->beta, rt[0]->y};
  if(nr > 1) g.xr[1] = rt[1]->x, r1 = Term{rt[1]->alpha, rt[1]->beta, rt[1]->y};
  if(cterm) g.xc = cterm->x, ct = Term{cterm->alpha, cterm->beta, cterm->y};
  if(nr == 1 && !cterm) return launch_gemv<1, false, false, false>(ctx, g, r0, r1, ct, "gemv_n");
  if(nr == 0 && cterm) return launch_gemv<0, true, false, false>(ctx, g, r0, r1, ct, "gemv_t");
  if(nr == 1 && cterm) return launch_gemv<1, true, false, false>(ctx, g, r0, r1, ct, "gemv_nt");
  return launch_gemv<2, false, false, false>(ctx, g, r0, r1, ct, "gemv_nn");
}

gbpoly_status gbpoly_gemv_f32(gbpoly_ctx* ctx, gbpoly_op op, int64_t rows, int64_t cols, float alpha, const float* A,
    int64_t lda, const float* x, float beta, float* y) {
  gbpoly_gemv_term t{op, alpha, beta, x, y};
  return gbpoly_gemv_pair_f32(ctx, rows, cols, A, lda, &t, 1);
}

gbpoly_status gbpoly_atax_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, const float* A, int64_t lda, const float* x,
    float* tmp, float* y) {
  gbpoly_status st = check_common(ctx, rows, cols, A, lda);
  if(st != GBPOLY_OK) return st;
  if((cols > 0 && (!x || !y)) || (rows > 0 && !tmp)) return fail(GBPOLY_ERR_INVALID, "vector: null pointer");
  if(rows == 0 || cols == 0) return GBPOLY_OK;  // empty sums: tmp and y unchanged
  const bool vec = (cols % 4 == 0) && (lda % 4 == 0) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
  const int chunks = int((cols + kTileCols - 1) / kTileCols);
  if(vec && chunks <= 8) {
    switch(chunks) {
    case 1: return launch_atax<1>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 2: return launch_atax<2>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 3: return launch_atax<3>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 4: return launch_atax<4>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 5: return launch_atax<5>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 6: return launch_atax<6>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    case 7: return launch_atax<7>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    default: return launch_atax<8>(ctx, A, lda, int(rows), int(cols), x, tmp, y);
    }
  }
  // wide or unaligned matrices: the two passes
  if((st = gbpoly_gemv_f32(ctx, GBPOLY_OP_N, rows, cols, 1.f, A, lda, x, 1.f, tmp)) != GBPOLY_OK) return st;
  return gbpoly_gemv_f32(ctx, GBPOLY_OP_T, rows, cols, 1.f, A, lda, tmp, 1.f, y);
}

gbpoly_status gbpoly_gesummv_f32(gbpoly_ctx* ctx, int64_t rows, int64_t cols, float alpha, const float* A,
    int64_t lda, const float* B, int64_t ldb, const float* x, float beta, float* tmp, float* y) {
  gbpoly_status st = check_common(ctx, rows, cols, A, lda);
  if(st != GBPOLY_OK) return st;
  if((st = check_common(ctx, rows, cols, B, ldb)) != GBPOLY_OK) return st;
  if((cols > 0 && !x) || (rows > 0 && (!tmp || !y))) return fail(GBPOLY_ERR_INVALID, "vector: null pointer");
  GemvArgs g{};
  g.A = A, g.lda = lda, g.B = B, g.ldb = ldb, g.rows = int(rows), g.cols = int(cols);
  g.xr[0] = x, g.xr[1] = x;
  return launch_gemv<2, false, true, true>(ctx, g, Term{1.f, 1.f, tmp}, Term{alpha, beta, y}, Term{}, "gesummv");
}

}  // extern "C"
