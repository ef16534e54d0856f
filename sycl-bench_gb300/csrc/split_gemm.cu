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
//   fp16x3    FP16  2      a0.b0 + a0.b1 + a1.b0 of x 2^e, one power-of-two
//                          2^e per 64x64 operand block (FP32's range)        22
//   fp8       E4M3  1      a0.b0, each operand with one scale per 128x128 block   4
// Two kernels per call:
//   * split_kernel (memory bound): writes the K-major term panels of an
//     operand into the context workspace (an MN-major operand transposed by
//     the register assignment), K padded with zeros to the k-block; for FP16
//     terms also each block's inverse scale;
//   * split_gemm_kernel: persistent (one CTA per SM walks 128 x BN tiles of
//     C), warp specialised, 384 threads:
//       warp 0      TMA producer: the term tiles of A (128 rows) and B (BN rows),
//                   128-byte rows (64 BF16 or 32 TF32 along K) with 128-byte
//                   swizzle, into a ring of STAGES shared-memory stages;
//       warp 1      allocates all 512 TMEM columns; one lane issues the
//                   products' tcgen05.mma (M=128, N=BN; K=16 BF16 or K=8 TF32)
//                   into one of NBUF TMEM chunk buffers (2 of 256 columns or
//                   4 of 128), restarting the accumulator every CH stages,
//                   and commits stages and chunks;
//       warps 4-11  epilogue (setmaxnreg 208): each warp owns 32 rows (its
//                   TMEM lane quarter) x BN/2 columns and sums the chunks in
//                   FP32 registers with round-to-nearest adds (scaled forms:
//                   times the chunk's left x right block factor), then writes
//                   C = alpha*acc + beta*C (through a per-warp staging tile,
//                   or, in the C-tile configurations, through TMA-loaded and
//                   TMA-stored boxes of C in shared memory).
//     CTA-pair configurations (cluster of two, cta_group::2) compute 256 x BN
//     tiles, each CTA staging 128 rows of A and BN/2 rows of B; when a
//     launch's last round of tiles would leave half the pairs or more idle,
//     its tiles run as two K halves on two pairs (the K-split tail).
//     The tensor core accumulates with truncation: over long K its error
//     grows with the number of MMA steps (measured 3.6e-6 normwise at K=512
//     for 24-bit operand splits, against 2.6e-7 for the same products summed
//     with round to nearest).  Each stage therefore starts a fresh TMEM
//     chunk, issues its cross products before its main product (only the
//     last BK/KMMA truncating steps see the full-size partial sum), and the
//     chunks are summed with round to nearest in registers.
//     syr2k's two products (A_i.B_j^T + B_i.A_j^T) alternate stage by stage
//     into the same accumulator.
// All mbarrier waits are bounded (gbpoly_internal.cuh).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "gbpoly_internal.cuh"
#include "umma.cuh"

namespace gbpoly {
namespace {

enum class Elem { BF16, TF32, E4M3, F16 };

// Instruction descriptor of an M x N MMA of element type E (FP32 accumulation).
template <Elem E, int M, int N>
constexpr uint32_t idesc_of() {
  if constexpr(E == Elem::E4M3)
    return umma::InstrDescE4M3<M, N>::value;
  else
    return umma::InstrDesc<M, N,
        E == Elem::BF16 ? umma::AbType::BF16 : (E == Elem::F16 ? umma::AbType::F16 : umma::AbType::TF32)>::value;
}

// CG_ = 2: a CTA pair (cluster of two) computes a (256 x BN) tile with
// cta_group::2 MMAs: each CTA holds 128 rows of the A tile and BN/2 rows of
// the B tile in its shared memory, and 128 rows x BN columns of the
// accumulator in its TMEM.
// CEPI_: the C tile of a CTA (128 x BN FP32) has its own shared-memory
// buffer, filled by TMA when the tile starts and written back by TMA stores
// (non-symmetric products with 16-byte-aligned C rows; no K-split tail).
template <Elem E, int TERMS, int NPROD, int BN_, int STAGES_, int ROW_ = 128, int CG_ = 1, bool CEPI_ = false>
struct Form {
  static constexpr Elem elem = E;
  static constexpr int CG = CG_;
  static constexpr bool CEPI = CEPI_;
  static constexpr int terms = TERMS, nprod = NPROD, BN = BN_, STAGES = STAGES_;
  static constexpr int BM_CTA = 128, BM = BM_CTA * CG;   // rows per CTA; rows of a (pair) tile
  static constexpr int BN_CTA = BN / CG;                 // B rows staged per CTA
  static constexpr int ROW = ROW_;                       // bytes of K per smem row (= swizzle width)
  static constexpr int esz = (E == Elem::BF16 || E == Elem::F16) ? 2 : (E == Elem::TF32 ? 4 : 1);
  static constexpr int BK = ROW / esz;                   // K elements per stage
  static constexpr int KMMA = 32 / esz;                  // K of one tcgen05.mma (32 bytes)
  // E4M3 operands carry one scale per 128 x 128 block, F16 terms one
  // power-of-two scale per 64 x 64 block: a stage (128 bytes of K) is exactly
  // one block along K, so each TMEM chunk has one scale per SCALE_ROWS rows
  // of either operand.
  static constexpr bool scaled = E == Elem::E4M3 || E == Elem::F16;
  static constexpr int SCALE_ROWS = E == Elem::F16 ? 64 : 128;
  static constexpr int A_TILE = BM_CTA * ROW, B_TILE = BN_CTA * ROW;
  static constexpr int STAGE = TERMS * (A_TILE + B_TILE);  // bytes per stage in each CTA
  static constexpr int STAGE_TX = CG * STAGE;              // bytes a stage's barrier waits for (both CTAs)
  static constexpr int EPI_STAGE = 8 * 32 * 33 * 4;  // epilogue staging, one 32x33 fp32 tile per warp
  static constexpr int C_BOX = 32 * 32 * 4;          // CEPI: one 32 x 32 FP32 box of C (128-byte swizzle)
  static constexpr int C_TILE = 8 * (BN / 64) * C_BOX;  // CEPI: 8 epilogue warps x HALF / 32 boxes
  // stages, barriers (256 bytes; CEPI: padded to 1 KB), epilogue staging or the C tile, alignment slack
  static constexpr int SMEM = CEPI ? STAGES * STAGE + 1024 + C_TILE + 1024 : STAGES * STAGE + 1024 + 256 + EPI_STAGE;
  // Accumulation: CH stage iterations per TMEM chunk (round-toward-zero
  // accumulation inside the tensor core stays short); chunks are summed in
  // FP32 registers, round to nearest, by the epilogue warps.  NBUF chunk
  // buffers in TMEM (all 512 columns: 2 of 256, 4 of 128) so the MMAs run
  // ahead of the epilogue, also across the C stores between two tiles.
  static constexpr int CH = 128 / ROW;
  static constexpr int NBUF = BN <= 128 ? 4 : 2;
  // TMEM allocations are powers of two (>= 32 columns); chunk buffer b
  // starts at column b * BUF_COLS
  static constexpr uint32_t TMEM_COLS = NBUF * BN <= 64 ? 64 : (NBUF * BN <= 128 ? 128 : (NBUF * BN <= 256 ? 256 : 512));
  static constexpr uint32_t BUF_COLS = TMEM_COLS / NBUF;
  static constexpr int HALF = BN / 2;  // columns per epilogue warp
  // Square tiles: symmetric updates compute the lower triangle of tiles and
  // mirror them.
  static constexpr bool MIRROR = BM == BN;
  static constexpr int THREADS = 384;  // warpgroup 0: producer, MMA; warpgroups 1-2: epilogue
  static constexpr uint32_t REGS_CTRL = 56, REGS_EPI = 208;
  static constexpr uint32_t IDESC = idesc_of<E, BM, BN>();
  static_assert(!scaled || (ROW == 128 && CH == 1), "one scale block per chunk");
  static_assert(CG == 1 || (CG == 2 && E != Elem::E4M3 && BN % 32 == 0), "CTA pairs: BF16, F16 and TF32 forms");
  static_assert(STAGE_TX == CG * STAGE, "pair stage bytes");
  static_assert(SMEM <= 232448, "shared memory");
  static_assert(TMEM_COLS <= 512 && BUF_COLS >= BN, "tensor memory");
  static_assert((2 * STAGES + 2 * NBUF + 1 + (CEPI ? 8 : 0)) * 8 + 4 <= 256, "barriers fit their 256 bytes");
  static_assert(!CEPI || (ROW == 128 && !scaled && CG == 2), "C-tile epilogue: CTA-pair 128-byte-row forms");
};

// Tile configurations per form (index = config id).  Config 0 is the default.
using FormTF32 = Form<Elem::TF32, 1, 1, 256, 4>;
using FormTF32_b = Form<Elem::TF32, 1, 1, 256, 8, 64>;
using FormTF32_c = Form<Elem::TF32, 1, 1, 128, 6>;
using FormBF16x3 = Form<Elem::BF16, 2, 3, 256, 2>;
using FormBF16x3_b = Form<Elem::BF16, 2, 3, 256, 4, 64>;
using FormBF16x3_c = Form<Elem::BF16, 2, 3, 128, 3>;
using FormTF32x3 = Form<Elem::TF32, 2, 3, 256, 2>;
using FormTF32x3_b = Form<Elem::TF32, 2, 3, 256, 4, 64>;
using FormTF32x3_c = Form<Elem::TF32, 2, 3, 128, 3>;
using FormBF16x6 = Form<Elem::BF16, 3, 6, 128, 2>;
using FormBF16x6_b = Form<Elem::BF16, 3, 6, 128, 4, 64>;
using FormBF16x6_c = Form<Elem::BF16, 3, 6, 256, 2, 64>;
// split-FP16 (fp16x3): the bf16x3 shapes with F16 terms and block scales
using FormF16x3 = Form<Elem::F16, 2, 3, 256, 2>;
using FormF16x3_c = Form<Elem::F16, 2, 3, 128, 3>;
using FormF16x3_p = Form<Elem::F16, 2, 3, 256, 3, 128, 2>;
using FormFP8 = Form<Elem::E4M3, 1, 1, 128, 6>;
using FormFP8_w = Form<Elem::E4M3, 1, 1, 256, 4>;  // 128 x 256 tiles: twice the MMA work per scaled chunk
// CTA-pair configurations (cluster of 2, 256 x 256 tiles)
using FormTF32_p = Form<Elem::TF32, 1, 1, 256, 6, 128, 2>;
using FormBF16x3_p = Form<Elem::BF16, 2, 3, 256, 3, 128, 2>;
using FormTF32x3_p = Form<Elem::TF32, 2, 3, 256, 3, 128, 2>;
using FormBF16x6_p = Form<Elem::BF16, 3, 6, 256, 2, 128, 2>;
// CTA pairs with 64-byte rows: more, shorter stages
using FormTF32_q = Form<Elem::TF32, 1, 1, 256, 12, 64, 2>;
using FormBF16x3_q = Form<Elem::BF16, 2, 3, 256, 6, 64, 2>;
using FormTF32x3_q = Form<Elem::TF32, 2, 3, 256, 6, 64, 2>;
using FormBF16x6_q = Form<Elem::BF16, 3, 6, 256, 4, 64, 2>;
// CTA pairs with the C tile in shared memory (TMA loads and stores of C,
// fewer pipeline stages): GEMMs whose K is too short to hide C's traffic
using FormTF32_t = Form<Elem::TF32, 1, 1, 256, 2, 128, 2, true>;
using FormBF16x3_t = Form<Elem::BF16, 2, 3, 256, 1, 128, 2, true>;
using FormTF32x3_t = Form<Elem::TF32, 2, 3, 256, 1, 128, 2, true>;
using FormBF16x6_t = Form<Elem::BF16, 3, 6, 256, 1, 128, 2, true>;

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
struct Term<Elem::F16> {
  using T = __half;
  __device__ static T round(float x) { return __float2half_rn(x); }
  __device__ static float widen(T x) { return __half2float(x); }
};
template <>
struct Term<Elem::TF32> {
  using T = float;
  __device__ static T round(float x) { return round_tf32(x); }
  __device__ static float widen(T x) { return x; }
};

// ------------------------------------------------------------- split pass --
// One 64 x 64 block of op(X) at (r0, k0) per CTA of 256 threads (or per
// iteration of a persistent CTA); every thread loads 16 values with 16-byte
// loads along the rows of X and converts 16 values:
//   K-major op(X) (op(X)[r][k] = X[r ld + k], rows contiguous in k):
//     split_load gives thread t elements [4 (t % 16), +4) of the block's rows
//     t / 16 + 16 e (e < 4); split_convert_kmajor writes their terms (8 bytes
//     of BF16 or FP16, 16 of TF32 per row and term: 128-byte row segments
//     per 16 threads).
//   MN-major op(X) (op(X)[r][k] = X[k ld + r]): split_load reads the block's
//     k rows of X the same way (thread t: r = 4 (t % 16) + j, k = t / 16 +
//     16 e), and mn_to_kmajor turns them through a 64 x 65 shared tile into
//     the K-major assignment, so the rest is the K-major path.
// Values outside R x K are zero, so the K padding of the panels is written
// with zeros.  Both convert the same way: terms by SplitTerms, an optional
// per-row transform first (RowXform).
//
// Rows of X that do not start on a 16-byte boundary (a
// leading dimension that is not a multiple of 4, or an offset base) are read
// with the aligned 16-byte loads that cover them: a row segment starting a
// floats (a < 4) past a boundary is covered by 17 chunks; lane q of a half
// warp (one row) loads chunk q, takes chunk q + 1 from its neighbour by a
// shuffle (lane 15 loads chunk 16 itself), and selects its four elements
// with two branch-free shift stages (by a & 1, then by a & 2).  Every chunk
// read holds at least one element of the matrix, so no read leaves the
// 16-byte granules of the matrix's own elements.
__device__ __forceinline__ void split_load(const float* __restrict__ X, int64_t ld, int k_major, int R, int K,
    int64_t r0, int64_t k0, float (&v)[16]) {
  const int tid = threadIdx.x;
  const int64_t r_lim = R - r0, k_lim = K - k0;
  const int64_t o0 = k_major ? r0 : k0, i0 = k_major ? k0 : r0;  // outer (strided) and inner (contiguous) origin
  const int out = tid >> 4, q = tid & 15;
  const bool whole = r_lim >= 64 && k_lim >= 64 && (ld & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0;
  if(whole) {
    const float* p = X + (o0 + out) * ld + i0 + 4 * q;
#pragma unroll
    for(int e = 0; e < 4; ++e) {
      const float4 x = *reinterpret_cast<const float4*>(p + e * 16 * ld);
      v[4 * e] = x.x, v[4 * e + 1] = x.y, v[4 * e + 2] = x.z, v[4 * e + 3] = x.w;
    }
    return;
  }
  const int64_t in_lim = k_major ? k_lim : r_lim, out_lim = k_major ? r_lim : k_lim;
  float4 c[4], x16[4];
  int al[4];
#pragma unroll
  for(int e = 0; e < 4; ++e) {  // all loads first
    const int o = out + 16 * e;
    const bool row_ok = o < out_lim;
    const float* row = X + (o0 + (row_ok ? o : 0)) * ld + i0;
    const int a = int((reinterpret_cast<uintptr_t>(row) >> 2) & 3);
    const float4* ch = reinterpret_cast<const float4*>(row - a);
    al[e] = a;
    c[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    x16[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    if(row_ok && max(4 * q - a, 0) < in_lim) c[e] = ch[q];          // holds row[max(4q - a, 0)]
    if(row_ok && q == 15 && a != 0 && 64 - a < in_lim) x16[e] = ch[16];  // holds row[64 - a]
  }
#pragma unroll
  for(int e = 0; e < 4; ++e) {
    float4 n;
    n.x = __shfl_down_sync(0xffffffffu, c[e].x, 1, 16);
    n.y = __shfl_down_sync(0xffffffffu, c[e].y, 1, 16);
    n.z = __shfl_down_sync(0xffffffffu, c[e].z, 1, 16);
    if(q == 15) n = x16[e];
    const int a = al[e];
    // w = c0.x c0.y c0.z c0.w n.x n.y n.z; element j of the thread is w[j + a]
    const bool s1 = a & 1, s2 = a & 2;
    const float u0 = s1 ? c[e].y : c[e].x, u1 = s1 ? c[e].z : c[e].y, u2 = s1 ? c[e].w : c[e].z;
    const float u3 = s1 ? n.x : c[e].w, u4 = s1 ? n.y : n.x, u5 = s1 ? n.z : n.y;
    float y[4] = {s2 ? u2 : u0, s2 ? u3 : u1, s2 ? u4 : u2, s2 ? u5 : u3};
    const bool row_ok = out + 16 * e < out_lim;
#pragma unroll
    for(int j = 0; j < 4; ++j) v[4 * e + j] = (row_ok && 4 * q + j < in_lim) ? y[j] : 0.f;
  }
}

// Terms of NV consecutive values: t[j] = round(x - t[0] - ... - t[j-1]).
// BF16: two values per conversion (cvt.rn.bf16x2.f32, the same round to
// nearest even as one at a time).
template <Elem E, int TERMS, int NV = 16>
struct SplitTerms {
  using T = typename Term<E>::T;
  __device__ static void run(const float* x, T (&t)[TERMS][NV]) {
#pragma unroll
    for(int i = 0; i < NV; ++i) {
      float rem = x[i];
#pragma unroll
      for(int j = 0; j < TERMS; ++j) {
        t[j][i] = Term<E>::round(rem);
        rem -= Term<E>::widen(t[j][i]);
      }
    }
  }
};
template <int TERMS, int NV>
struct SplitTerms<Elem::BF16, TERMS, NV> {
  __device__ static void run(const float* x, __nv_bfloat16 (&t)[TERMS][NV]) {
#pragma unroll
    for(int i = 0; i < NV; i += 2) {
      float a = x[i], b = x[i + 1];
#pragma unroll
      for(int j = 0; j < TERMS; ++j) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        t[j][i] = h.x;
        t[j][i + 1] = h.y;
        a -= __low2float(h);
        b -= __high2float(h);
      }
    }
  }
};

// K-major operands (op(X) rows contiguous in X) need no transposition: each
// thread converts the values split_load gave it (rows t / 16 + 16 e, k
// elements [4 (t % 16), +4)) straight into the panels, the same arithmetic as
// split_convert (row transform included), without the shared tile.
template <Elem E, int TERMS>
__device__ __forceinline__ void split_convert_kmajor(const float (&v)[16], typename Term<E>::T* __restrict__ out,
    int64_t panel_stride, int R, int Kp, int64_t r0, int64_t k0, RowXform xf = RowXform{}, int K = 0) {
  using T = typename Term<E>::T;
  const int tid = threadIdx.x;
  const int rr = tid >> 4, kc = 4 * (tid & 15);
#pragma unroll
  for(int e = 0; e < 4; ++e) {
    const int64_t r = r0 + rr + 16 * e;
    if(r >= R) continue;
    float x[4] = {v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]};
    if(xf.mean) {
      const float m = xf.mean[r], sd = xf.sd ? xf.sd[r] : 1.f;
#pragma unroll
      for(int i = 0; i < 4; ++i) {
        float y = x[i] - m;
        if(xf.sd) y = (y / xf.div) / sd;
        x[i] = k0 + kc + i < K ? y : 0.f;
      }
    }
    __align__(16) T t[TERMS][4];
    SplitTerms<E, TERMS, 4>::run(x, t);
#pragma unroll
    for(int j = 0; j < TERMS; ++j) {
      T* dst = out + j * panel_stride + r * Kp + k0 + kc;
      if constexpr(sizeof(T) == 2)
        *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(t[j]);
      else
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(t[j]);
    }
  }
}

// An MN-major block as split_load gives it (k_major = 0: thread t holds the
// elements r = 4 (t % 16) + j, k = t / 16 + 16 e, from 16-byte loads along
// the rows of X) turned through a 64 x 65 shared tile into the K-major
// assignment (rows t / 16 + 16 e, k in [4 (t % 16), +4)), so the transform,
// the block scale and the panel stores are the K-major path's: 128-byte row
// segments per 16 threads.  All 256 threads; the first barrier lets a
// persistent CTA reuse the tile for its next block.
__device__ __forceinline__ void mn_to_kmajor(const float (&v)[16], float (&w)[16]) {
  __shared__ float tile[64][65];
  const int tid = threadIdx.x, q = tid & 15, o = tid >> 4;
  __syncthreads();
#pragma unroll
  for(int e = 0; e < 4; ++e)
#pragma unroll
    for(int j = 0; j < 4; ++j) tile[4 * q + j][o + 16 * e] = v[4 * e + j];
  __syncthreads();
#pragma unroll
  for(int e = 0; e < 4; ++e)
#pragma unroll
    for(int i = 0; i < 4; ++i) w[4 * e + i] = tile[o + 16 * e][4 * q + i];
}

// The row transform of split_convert_kmajor applied in place to a thread's
// values (same arithmetic), for the F16 form, whose block scale is taken
// after the transform.
__device__ __forceinline__ void xform_kmajor(float (&v)[16], int R, int64_t r0, int64_t k0, const RowXform& xf, int K) {
  if(!xf.mean) return;
  const int tid = threadIdx.x;
  const int rr = tid >> 4, kc = 4 * (tid & 15);
#pragma unroll
  for(int e = 0; e < 4; ++e) {
    const int64_t r = r0 + rr + 16 * e;
    if(r >= R) continue;
    const float m = xf.mean[r], sd = xf.sd ? xf.sd[r] : 1.f;
#pragma unroll
    for(int i = 0; i < 4; ++i) {
      float y = v[4 * e + i] - m;
      if(xf.sd) y = (y / xf.div) / sd;
      v[4 * e + i] = k0 + kc + i < K ? y : 0.f;
    }
  }
}

// Power-of-two scale s of a 64 x 64 block for F16 terms (all 256 threads):
// with the block maximum m = f 2^ex (f in [0.5, 1)), s = 2^(15 - ex) puts
// m s in [2^14, 2^15), so the hi term stays below FP16's largest finite
// value (65504) and the lo term, about 2^-11 of hi, stays in FP16's normal
// range for every element within 2^-18 of the block maximum.  Scaling by a
// power of two is exact; 1/s (also exact) goes to *inv_out for the
// epilogue.  The maximum is over the finite elements (an infinity or NaN
// stays one and leaves the block's other elements scaled); an all-zero
// block gives s = 1.
// red: 8 words of shared memory (a loop over blocks alternates two sets, so
// that a warp ahead by one block never overwrites words still being read).
__device__ __forceinline__ float block_pow2_scale(const float (&v)[16], float* inv_out, float* red) {
  float m = 0.f;
#pragma unroll
  for(int i = 0; i < 16; ++i) m = fabsf(v[i]) < INFINITY ? fmaxf(m, fabsf(v[i])) : m;  // finite elements
#pragma unroll
  for(int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = red[0];
#pragma unroll
  for(int w = 1; w < 8; ++w) m = fmaxf(m, red[w]);
  const uint32_t bits = __float_as_uint(m);
  int e = 0;
  if(m > 0.f && (bits & 0x7f800000u) != 0x7f800000u) {
    const int biased = int((bits >> 23) & 0xffu);
    const int ex = biased == 0 ? -125 : biased - 126;  // m = f 2^ex, f in [0.5, 1) (subnormal m: below that)
    e = min(max(15 - ex, -120), 120);
  }
  if(threadIdx.x == 0) *inv_out = __uint_as_float(uint32_t(127 - e) << 23);
  return __uint_as_float(uint32_t(127 + e) << 23);
}

// panel[t][r][k] (r < R, k < Kp) = term t of op(X)[r][k] for k < K, 0 beyond,
// op(X)[r][k] = X[r*ld + k] (k_major) or X[k*ld + r].  Panels are Kp-strided
// and `panel_stride` elements apart.  One 64 x 64 block per CTA.  F16 terms:
// the block is scaled by a power of two first (block_pow2_scale) and its
// inverse scale stored at inv_scale[blockIdx.y * gridDim.x + blockIdx.x].
template <Elem E, int TERMS>
__global__ void __launch_bounds__(256) split_kernel(const float* __restrict__ X, int64_t ld, int k_major, int R, int K,
    int Kp, typename Term<E>::T* __restrict__ out, int64_t panel_stride, RowXform xf, float* __restrict__ inv_scale) {
  const int64_t r0 = int64_t(blockIdx.y) * 64, k0 = int64_t(blockIdx.x) * 64;
  float v[16];
  if(k_major) {
    split_load(X, ld, 1, R, K, r0, k0, v);
  } else {
    float t[16];
    split_load(X, ld, 0, R, K, r0, k0, t);
    mn_to_kmajor(t, v);
  }
  if constexpr(E == Elem::F16) {
    xform_kmajor(v, R, r0, k0, xf, K);
    __shared__ float red[8];
    const float s = block_pow2_scale(v, inv_scale + int64_t(blockIdx.y) * gridDim.x + blockIdx.x, red);
#pragma unroll
    for(int i = 0; i < 16; ++i) v[i] *= s;
    split_convert_kmajor<E, TERMS>(v, out, panel_stride, R, Kp, r0, k0);
  } else {
    split_convert_kmajor<E, TERMS>(v, out, panel_stride, R, Kp, r0, k0, xf, K);
  }
}

// One operand of a grouped call; its 64 x 64 blocks are listed in the
// plan's block table.
struct SplitJob {
  const float* X;
  int64_t ld;
  int k_major, R, K, Kp;
  void* out;
  int64_t panel_stride;  // elements
  float* scale;          // F16 terms: inverse block scales, [row block][Kp / 64]
};

// Grouped split pass: persistent CTAs walk the blocks in a grid-stride loop
// (block b, b + gridDim.x, ...: the blocks in flight at a time are
// neighbours in memory, as in a one-block-per-CTA launch); blocks[b] =
// (job, row block, k block) is written by the plan.  The next block's table
// entry and job are read while the current block is loaded and converted, so
// a block's data loads wait on one memory latency, not three; those are
// covered by the 32 resident warps per SM, each with 16 loads in flight.
template <Elem E, int TERMS>
__global__ void __launch_bounds__(256, 4) grouped_split_kernel(const SplitJob* __restrict__ jobs,
    const int4* __restrict__ blocks, int nblocks) {
  using T = typename Term<E>::T;
  int b = blockIdx.x;
  if(b >= nblocks) return;
  int4 bl = blocks[b];
  SplitJob j = jobs[bl.x];
  int4 bl_next = b + int(gridDim.x) < nblocks ? blocks[b + gridDim.x] : make_int4(0, 0, 0, 0);
  __shared__ float red[2][8];  // F16: block maxima, alternating sets
  for(int iter = 0;; ++iter) {
    const int64_t r0 = int64_t(bl.y) * 64, k0 = int64_t(bl.z) * 64;
    float v[16];
    split_load(j.X, j.ld, j.k_major, j.R, j.K, r0, k0, v);
    const int nb = b + int(gridDim.x);
    const SplitJob jn = jobs[bl_next.x];  // in flight with this block's loads
    const int4 bl_after = nb + int(gridDim.x) < nblocks ? blocks[nb + gridDim.x] : make_int4(0, 0, 0, 0);
    if(!j.k_major) {
      float t[16];
#pragma unroll
      for(int i = 0; i < 16; ++i) t[i] = v[i];
      mn_to_kmajor(t, v);
    }
    if constexpr(E == Elem::F16) {
      const float s = block_pow2_scale(v, j.scale + int64_t(bl.y) * (j.Kp / 64) + bl.z, red[iter & 1]);
#pragma unroll
      for(int i = 0; i < 16; ++i) v[i] *= s;
    }
    split_convert_kmajor<E, TERMS>(v, static_cast<T*>(j.out), j.panel_stride, j.R, j.Kp, r0, k0);
    if(nb >= nblocks) break;
    b = nb;
    bl = bl_next;
    j = jn;
    bl_next = bl_after;
  }
}

// ---------------------------------------------------------- FP8 quantize --
// 128 x 128 blocks of op(X) (rows x K, zero beyond R and K), walked by
// persistent CTAs of 512 threads (two per SM), one block at a time: scale = max|x| / 448 (1 for an all-zero block),
// q = e4m3(x / scale) with saturation, written K-major into out[R][Kp];
// scale into scales[row block][Kp / 128].  One launch quantises both
// operands of a contraction (blocks of the first, then of the second).  No
// shared-memory tile: every thread keeps 32 values of the block in
// registers, coalesced in both layouts:
//   K-major op(X) (rows contiguous in k): warp w holds rows 8w .. 8w + 7 of
//     the block, lane l the four k values [4l, 4l + 4) of each (16-byte
//     loads when the rows are 16-byte aligned and the block is whole in K),
//     and writes their four E4M3 bytes per row;
//   MN-major op(X) (op(X)[r][k] = X[k][r]): warp w holds the 32 x 32
//     sub-block k in [32 (w / 4), +32), r in [32 (w % 4), +32); lane l reads
//     column r = 32 (w % 4) + l down the 32 k (each load a 128-byte row
//     segment across the warp), which is 32 consecutive k of output row r:
//     the transpose happens in the register assignment, and the lane writes
//     its row's 32 bytes.
// Only the block maximum crosses warps (one shuffle reduction, 16 words of
// shared memory).
struct QuantJob {
  const float* X;
  int64_t ld;
  int k_major, R, K, Kp, kb;  // kb: 128-blocks along K
  uint8_t* out;
  float* scales;
};

__device__ __forceinline__ uint16_t e4m3x2(float a, float b) {
  return __nv_cvt_float2_to_fp8x2(make_float2(a, b), __NV_SATFINITE, __NV_E4M3);
}

__global__ void __launch_bounds__(512, 2) quantize_e4m3_kernel(const QuantJob ja, const QuantJob jb, int blocks_a,
    int nblocks) {
  __shared__ float red[16];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for(int blk = blockIdx.x; blk < nblocks; blk += gridDim.x) {
    const bool first = blk < blocks_a;
    const QuantJob& j = first ? ja : jb;
    const int local = first ? blk : blk - blocks_a;
    const int rb = local / j.kb, kbi = local % j.kb;
    const int64_t r0 = int64_t(rb) * 128, k0 = int64_t(kbi) * 128;
    float x[32];
    if(j.k_major) {
      const int64_t kc = k0 + 4 * lane;
      const bool vec = (j.ld & 3) == 0 && (reinterpret_cast<uintptr_t>(j.X) & 15) == 0 && k0 + 128 <= j.K;
#pragma unroll
      for(int i = 0; i < 8; ++i) {
        const int64_t r = r0 + 8 * warp + i;
        const float* p = j.X + r * j.ld + kc;
        if(r < j.R && vec) {
          const float4 f = *reinterpret_cast<const float4*>(p);
          x[4 * i] = f.x, x[4 * i + 1] = f.y, x[4 * i + 2] = f.z, x[4 * i + 3] = f.w;
        } else {
#pragma unroll
          for(int c = 0; c < 4; ++c) x[4 * i + c] = (r < j.R && kc + c < j.K) ? p[c] : 0.f;
        }
      }
    } else {
      const int64_t rr = r0 + 32 * (warp & 3) + lane, kk = k0 + 32 * (warp >> 2);
      const float* p = j.X + kk * j.ld + rr;
#pragma unroll
      for(int i = 0; i < 32; ++i) x[i] = (rr < j.R && kk + i < j.K) ? p[int64_t(i) * j.ld] : 0.f;
    }
    float amax = 0.f;
#pragma unroll
    for(int i = 0; i < 32; ++i) amax = fmaxf(amax, fabsf(x[i]));
#pragma unroll
    for(int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if(lane == 0) red[warp] = amax;
    __syncthreads();
    float m = red[0];
#pragma unroll
    for(int w = 1; w < 16; ++w) m = fmaxf(m, red[w]);
    const float scale = m > 0.f ? m / 448.f : 1.f;
    const float inv = 1.f / scale;
    if(tid == 0) j.scales[int64_t(rb) * (j.Kp / 128) + kbi] = scale;
    if(j.k_major) {
#pragma unroll
      for(int i = 0; i < 8; ++i) {
        const int64_t r = r0 + 8 * warp + i;
        if(r >= j.R) continue;
        const uint32_t q = uint32_t(e4m3x2(x[4 * i] * inv, x[4 * i + 1] * inv)) |
                           (uint32_t(e4m3x2(x[4 * i + 2] * inv, x[4 * i + 3] * inv)) << 16);
        *reinterpret_cast<uint32_t*>(j.out + r * j.Kp + k0 + 4 * lane) = q;
      }
    } else {
      const int64_t rr = r0 + 32 * (warp & 3) + lane;
      if(rr < j.R) {
        __align__(16) uint16_t q[16];
#pragma unroll
        for(int i = 0; i < 16; ++i) q[i] = e4m3x2(x[2 * i] * inv, x[2 * i + 1] * inv);
        uint4* dst = reinterpret_cast<uint4*>(j.out + rr * j.Kp + k0 + 32 * (warp >> 2));
        dst[0] = reinterpret_cast<const uint4*>(q)[0];
        dst[1] = reinterpret_cast<const uint4*>(q)[1];
      }
    }
    __syncthreads();  // red[] is read by every thread before the next block writes it
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

// What every warp role needs to know about one output tile.
struct TileInfo {
  int m0, n0, M, N, Kp, npair;
  float alpha, beta;
  float* C;
  int64_t ldc;
  const ProductMaps* maps;  // [npair]
  // Scaled forms (E4M3, F16): per pairing, scales of the left and right
  // operand blocks, [row block][k block] with kt k blocks per row block
  const float* sl[2];
  const float* sr[2];
  int kt;
  bool mirror;  // symmetric update, tile strictly below the diagonal: also write its transpose
};

// One contraction: tiles in grouped raster order, tensor maps in the
// kernel's parameter space.
template <int BM, int BN>
struct SingleSched {
  GemmMaps maps;
  int npair, M, N, Kp;
  float alpha, beta;
  float* C;
  int64_t ldc;
  const float* sl[2] = {nullptr, nullptr};
  const float* sr[2] = {nullptr, nullptr};
  int kt = 0;  // scaled forms: scale blocks along K (a row of the scale tables)
  // Symmetric updates (syrk, syr2k: the product is symmetric, M == N, BM == BN):
  // only tiles on or below the diagonal are computed; the ones below it also
  // store their transpose.
  bool lower = false;
  // Split tail (CTA pairs): when the last round of tiles would leave half the
  // clusters or more idle, each of its tiles becomes two units of half the
  // K iterations each, run by two clusters in that round.  The second half
  // (role 2, iterations [split_it, end)) stores its sums in partial[slot]
  // and counts its epilogue warps in flags[slot]; the first half (role 1,
  // [0, split_it)) waits for all of them (bounded), adds them to its own
  // sums and writes C.  units == 0: one unit per tile.
  int units = 0, full_tiles = 0, split_it = 0;
  float* partial = nullptr;  // [slot][CTA of the pair][128 rows][BN columns]
  int* flags = nullptr;      // [slot], zero at launch
  CUtensorMap cmap;          // C-tile epilogue forms: C (M x N, boxes of 32 x 32, 128-byte swizzle)
  __device__ int count() const {
    const int tm = (M + BM - 1) / BM, tn = (N + BN - 1) / BN;
    return lower ? tm * (tm + 1) / 2 : tm * tn;
  }
  __device__ int unit_count() const { return units ? units : count(); }
  // unit u -> tile, role (0 whole tile, 1 first K half, 2 second K half),
  // tail slot.  The half that stores its sums takes the lower unit (and
  // cluster) index of the two, the half that waits for them the higher.
  __device__ void unit(int u, int& t, int& role, int& slot) const {
    if(units == 0 || u < full_tiles) {
      t = u, role = 0, slot = 0;
      return;
    }
    const int v = u - full_tiles;
    t = full_tiles + v / 2, role = 2 - (v & 1), slot = v / 2;
  }
  __device__ TileInfo tile(int t) const {
    int tm, tn;
    if(lower) {  // row-major walk of the lower triangle: t = tm (tm + 1) / 2 + tn
      tm = int((sqrtf(8.f * float(t) + 1.f) - 1.f) * 0.5f);
      while(tm * (tm + 1) / 2 > t) --tm;
      while((tm + 1) * (tm + 2) / 2 <= t) ++tm;
      tn = t - tm * (tm + 1) / 2;
    } else {
      tile_coords(t, (M + BM - 1) / BM, (N + BN - 1) / BN, tm, tn);
    }
    return TileInfo{tm * BM, tn * BN, M, N, Kp, npair, alpha, beta, C, ldc, maps.p, {sl[0], sl[1]}, {sr[0], sr[1]},
        kt, lower && tm != tn};
  }
};

// A group of independent contractions (problem table and tensor maps in
// global memory), tiles of all problems in one list ordered by decreasing K.
struct GroupProblem {
  int M, N, Kp, pad;
  float alpha, beta;
  float* C;
  int64_t ldc;
  const float* sa;  // F16 terms: inverse block scales of A and B, [row block][Kp / 64]
  const float* sb;
};
template <int BM, int BN>
struct GroupedSched {
  const GroupProblem* probs;
  const ProductMaps* maps;  // one per problem
  const int4* tiles;        // (problem, tile_m, tile_n, 0)
  int ntiles;
  __device__ int count() const { return ntiles; }
  __device__ int unit_count() const { return ntiles; }
  int split_it = 0;
  float* partial = nullptr;
  int* flags = nullptr;
  __device__ void unit(int u, int& t, int& role, int& slot) const { t = u, role = 0, slot = 0; }
  __device__ TileInfo tile(int t) const {
    const int4 e = tiles[t];
    const GroupProblem p = probs[e.x];
    return TileInfo{e.y * BM, e.z * BN, p.M, p.N, p.Kp, 1, p.alpha, p.beta, p.C, p.ldc, maps + e.x, {p.sa, p.sa},
        {p.sb, p.sb}, p.Kp / 64, false};
  }
};

// Prefetch into L2 the C lines an epilogue warp (lane quarter q, column half
// h) reads for tile t: its 32 rows x HALF columns, and their mirror.
template <class F>
__device__ __forceinline__ void prefetch_c_warp(const TileInfo& t, uint32_t rank, int q, int h, int lane) {
  constexpr int segs = F::HALF / 32;  // 128-byte segments per row
  const int row0 = t.m0 + int(rank) * F::BM_CTA + 32 * q, col0 = t.n0 + h * F::HALF;
#pragma unroll
  for(int p = 0; p < segs; ++p) {
    const int l = lane + 32 * p, r = row0 + l / segs, n = col0 + 32 * (l % segs);
    if(r < t.M && n < t.N) prefetch_l2(t.C + int64_t(r) * t.ldc + n);
    if(F::MIRROR && t.mirror && col0 + l < t.N && row0 < t.M) prefetch_l2(t.C + int64_t(col0 + l) * t.ldc + row0);
  }
}

template <class F, class S>
__global__ void __launch_bounds__(F::THREADS, 1) split_gemm_kernel(const __grid_constant__ S sched, int* err) {
  extern __shared__ __align__(1024) char smem_raw[];
  char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + F::STAGES * F::STAGE);
  uint64_t* empty = full + F::STAGES;
  uint64_t* chunk_full = empty + F::STAGES;     // [NBUF]
  uint64_t* chunk_empty = chunk_full + F::NBUF;  // [NBUF]
  uint64_t* drain = chunk_empty + F::NBUF;
  uint64_t* cbar = drain + 1;  // C-tile epilogue: one barrier per epilogue warp for its C boxes
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1 + (F::CEPI ? 8 : 0));
  float(*epi_stage)[33] = reinterpret_cast<float(*)[33]>(smem + F::STAGES * F::STAGE + 256);  // 8 warps x [32][33]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int units = sched.unit_count();
  // CTA pairs: tiles are walked per cluster; rank 0 issues the MMAs and owns
  // the stage barriers, both CTAs load their halves and run the epilogue on
  // their 128 rows.
  const uint32_t rank = F::CG == 2 ? cluster_ctarank() : 0u;
  const int first_tile = F::CG == 2 ? int(cluster_id_x()) : int(blockIdx.x);
  const int tile_step = F::CG == 2 ? int(cluster_count_x()) : int(gridDim.x);

  if(threadIdx.x == 0) {
    for(int s = 0; s < F::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for(int b = 0; b < F::NBUF; ++b) {
      mbar_init(&chunk_full[b], 1);
      mbar_init(&chunk_empty[b], 8 * F::CG);  // one arrival per epilogue warp of the pair
    }
    mbar_init(drain, 1);
    if constexpr(F::CEPI)
      for(int w = 0; w < 8; ++w) mbar_init(&cbar[w], 1);
    fence_mbar_init();
  }
  if(warp == 1) {
    if constexpr(F::CG == 2) {
      umma::tmem_alloc_pair(tmem_slot, F::TMEM_COLS);
      umma::tmem_relinquish_pair();
    } else {
      umma::tmem_alloc(tmem_slot, F::TMEM_COLS);
      umma::tmem_relinquish();
    }
  }
  umma::fence_before_sync();
  if constexpr(F::CG == 2)
    cluster_sync();  // both CTAs' barriers initialised before any remote arrival
  else
    __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *tmem_slot;

  if(warp < 4) {
    umma::regs_decrease<F::REGS_CTRL>();
    if(warp == 0 && lane == 0) {
      // ---------------------------------------------------------- producer
      int g = 0;  // global stage iteration across tiles
      bool ok = true;
      for(int u = first_tile; u < units && ok; u += tile_step) {
        int tile, role, slot;
        sched.unit(u, tile, role, slot);
        const TileInfo ti = sched.tile(tile);
        const int m0 = ti.m0 + int(rank) * F::BM_CTA, n0 = ti.n0 + int(rank) * F::BN_CTA, npair = ti.npair;
        const int iters = (ti.Kp / F::BK) * npair;
        const int it0 = role == 2 ? sched.split_it : 0, it1 = role == 1 ? sched.split_it : iters;
        for(int it = it0; it < it1; ++it, ++g) {
          const int s = g % F::STAGES;
          if(g >= F::STAGES && !mbar_wait(&empty[s], ((g / F::STAGES) - 1) & 1, err, kDevErrEmptyWait)) {
            ok = false;
            break;
          }
          const ProductMaps& pm = ti.maps[it % npair];
          const int k0 = (it / npair) * F::BK;
          char* st = smem + s * F::STAGE;
          if constexpr(F::CG == 2) {
            // both CTAs' boxes complete on the first CTA's barrier, which expects the pair's bytes
            const uint32_t bar = cluster_map(&full[s], 0);
            if(rank == 0) mbar_arrive_expect_tx(&full[s], F::STAGE_TX);
#pragma unroll
            for(int t = 0; t < F::terms; ++t) {
              tma_load_2d_pair(st + t * F::A_TILE, &pm.l[t], bar, k0, m0);
              tma_load_2d_pair(st + F::terms * F::A_TILE + t * F::B_TILE, &pm.r[t], bar, k0, n0);
            }
          } else {
            mbar_arrive_expect_tx(&full[s], F::STAGE);
#pragma unroll
            for(int t = 0; t < F::terms; ++t) {
              tma_load_2d(st + t * F::A_TILE, &pm.l[t], &full[s], k0, m0);
              tma_load_2d(st + F::terms * F::A_TILE + t * F::B_TILE, &pm.r[t], &full[s], k0, n0);
            }
          }
        }
      }
      // do not leave while copies into shared memory are in flight: the
      // first CTA's barriers count the copies of both CTAs of a pair, and the
      // second CTA leaves only after the pair's final cluster barrier
      if(rank == 0)
        for(int h = max(0, g - F::STAGES); h < g; ++h)
          if(!mbar_wait(&full[h % F::STAGES], (h / F::STAGES) & 1, err, kDevErrDrainWait)) break;
    } else if(warp == 1 && lane == 0 && rank == 0) {
      // ------------------------------------------------------- MMA issue
      int g = 0, chunk = 0;
      bool ok = true;
      for(int u = first_tile; u < units && ok; u += tile_step) {
        int tile, role, slot;
        sched.unit(u, tile, role, slot);
        const TileInfo ti = sched.tile(tile);
        const int iters = (ti.Kp / F::BK) * ti.npair;
        const int it0 = role == 2 ? sched.split_it : 0, it1 = role == 1 ? sched.split_it : iters;
        for(int it = it0; it < it1 && ok; ++it, ++g) {
          const int b = chunk % F::NBUF;
          if(it % F::CH == 0) {
            // the epilogue must have drained this chunk buffer (used NBUF chunks ago)
            if(chunk >= F::NBUF && !mbar_wait(&chunk_empty[b], ((chunk / F::NBUF) - 1) & 1, err, kDevErrMmaWait)) {
              ok = false;
              break;
            }
            umma::fence_after_sync();
          }
          const int s = g % F::STAGES;
          if(!mbar_wait(&full[s], (g / F::STAGES) & 1, err, kDevErrFullWait)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const uint32_t d = tmem + uint32_t(b) * F::BUF_COLS;
          const uint32_t a_base = smem_u32(smem + s * F::STAGE);
          const uint32_t b_base = a_base + F::terms * F::A_TILE;
          // Issue order: every cross product (p >= 1) of the stage first, the
          // main product (p = 0) last, so the truncating accumulation runs on
          // a small partial sum for all but the last BK/KMMA steps.
          constexpr int KSTEPS = F::BK / F::KMMA;
#pragma unroll
          for(int q = 0; q < F::nprod * KSTEPS; ++q) {
            const int p = (q / KSTEPS + 1) % F::nprod;
            const int k = q % KSTEPS;
            const uint32_t off = k * 32;  // 32 bytes of K per MMA
            const uint64_t da = umma::desc_k<F::ROW>(a_base + prod_a(p) * F::A_TILE + off);
            const uint64_t db = umma::desc_k<F::ROW>(b_base + prod_b(p) * F::B_TILE + off);
            const uint32_t acc = (it % F::CH != 0 || q > 0) ? 1u : 0u;
            if constexpr(F::CG == 2) {
              if constexpr((F::elem == Elem::BF16 || F::elem == Elem::F16))
                umma::mma_f16_pair(d, da, db, F::IDESC, acc);
              else
                umma::mma_tf32_pair(d, da, db, F::IDESC, acc);
            } else if constexpr((F::elem == Elem::BF16 || F::elem == Elem::F16)) {
              umma::mma_f16(d, da, db, F::IDESC, acc);
            } else if constexpr(F::elem == Elem::TF32) {
              umma::mma_tf32(d, da, db, F::IDESC, acc);
            } else {
              umma::mma_f8(d, da, db, F::IDESC, acc);
            }
          }
          // stage s is free once these MMAs have read it (in both CTAs of a pair)
          if constexpr(F::CG == 2)
            umma::commit_pair(&empty[s], 0x3);
          else
            umma::commit(&empty[s]);
          if(it % F::CH == F::CH - 1 || it == it1 - 1) {
            // chunk complete in TMEM buffer b
            if constexpr(F::CG == 2)
              umma::commit_pair(&chunk_full[b], 0x3);
            else
              umma::commit(&chunk_full[b]);
            ++chunk;
          }
        }
      }
      // every MMA issued by this thread has completed
      if constexpr(F::CG == 2)
        umma::commit_pair(drain, 0x1);
      else
        umma::commit(drain);
      mbar_wait(drain, 0, err, kDevErrDrainWait);
    }
  } else {
    // ------------------------------------------------------------- epilogue
    umma::regs_increase<F::REGS_EPI>();
    const int q = warp & 3;          // TMEM lane quarter of this warp
    const int h = (warp - 4) >> 2;   // column half
    float acc[F::HALF];
    int chunk = 0;
    bool ok = true;
    // C-tile epilogue: this warp's HALF / 32 boxes of C, loads and stores issued so far
    char* const cbox = smem + F::STAGES * F::STAGE + 1024 + (warp - 4) * (F::HALF / 32) * F::C_BOX;
    int c_loads = 0, c_stores = 0;
    // chunk buffers are released on the first CTA's barrier (MMAs are issued there)
    static_assert(F::CG == 1 || F::NBUF == 2, "CTA pairs: two chunk buffers");
    const uint32_t chunk_empty_pair[2] = {F::CG == 2 ? cluster_map(&chunk_empty[0], 0) : 0u,
        F::CG == 2 ? cluster_map(&chunk_empty[1], 0) : 0u};
    for(int u = first_tile; u < units && ok; u += tile_step) {
      int tile, role, slot;
      sched.unit(u, tile, role, slot);
      const TileInfo ti = sched.tile(tile);
      const int M = ti.M, N = ti.N;
      const float alpha = ti.alpha, beta = ti.beta;
      const int64_t ldc = ti.ldc;
      const int iters = (ti.Kp / F::BK) * ti.npair;
      const int it0 = role == 2 ? sched.split_it : 0, it1 = role == 1 ? sched.split_it : iters;
      const int chunks = (it1 - it0 + F::CH - 1) / F::CH;
      const int nbase = ti.n0 + h * F::HALF;
      const int crow = ti.m0 + int(rank) * F::BM_CTA + 32 * q;
      if constexpr(F::CEPI) {
        // this tile's C into the warp's boxes while the MMAs run (once the
        // previous tile's stores have read them)
        if(beta != 0.f) {
          if(lane == 0) {
            if(c_stores > 0) bulk_wait_read_all();
            mbar_arrive_expect_tx(&cbar[warp - 4], (F::HALF / 32) * F::C_BOX);
#pragma unroll
            for(int j = 0; j < F::HALF / 32; ++j)
              tma_load_2d(cbox + j * F::C_BOX, &sched.cmap, &cbar[warp - 4], nbase + 32 * j, crow);
          }
          ++c_loads;
        }
      }
      // Scaled forms (E4M3, F16): chunk c (stage iteration it0 + c, CH = 1)
      // is multiplied by the factor of its left row block and right column
      // block, for each of the NCB blocks the warp's columns span.  Lane t
      // computes the factors of chunk 32 g + t for a whole group g of 32
      // chunks, one group ahead (its loads then have 32 chunks to land), and
      // every chunk takes its factors from lane c % 32 by shuffle: two scale
      // loads per lane per 32 chunks, not per thread per chunk.  Rows and
      // columns past the matrix edge, whose sums are not stored, read the
      // last block's scales (the tables hold the blocks that exist).
      constexpr int NCB = F::scaled && F::HALF > F::SCALE_ROWS ? F::HALF / F::SCALE_ROWS : 1;
      // factors of the current group's and the next group's chunk at this
      // lane: x alone, or x then y when one factor would leave FP32's range
      float fx[NCB], fy[NCB], nx[NCB], ny[NCB];
      auto load_group = [&](int g, float(&x)[NCB], float(&y)[NCB]) {
        const int cc = 32 * g + lane;
#pragma unroll
        for(int cb = 0; cb < NCB; ++cb) x[cb] = 1.f, y[cb] = 1.f;
        if(cc >= chunks) return;
        const int it = it0 + cc;
        const bool second = ti.npair == 2 && (it & 1);  // syr2k: iterations alternate the two pairings
        const int kb = ti.npair == 2 ? it >> 1 : it;
        const float* sl = second ? ti.sl[1] : ti.sl[0];  // selects, not indexing: keeps TileInfo in registers
        const float* sr = second ? ti.sr[1] : ti.sr[0];
        const int srow = min(crow, M - 1) / F::SCALE_ROWS;
        const float l = sl[srow * ti.kt + kb];
#pragma unroll
        for(int cb = 0; cb < NCB; ++cb) {
          const float r = sr[(min(nbase + F::SCALE_ROWS * cb, N - 1) / F::SCALE_ROWS) * ti.kt + kb];
          if constexpr(F::elem == Elem::F16) {
            // l = 2^-ea, r = 2^-eb with |ea|, |eb| <= 120: the factor
            // 2^-(ea + eb) is a normal float, or else two halves of it are
            const int e = int((__float_as_uint(l) >> 23) & 0xffu) + int((__float_as_uint(r) >> 23) & 0xffu) - 254;
            const int e1 = e >= -126 && e <= 127 ? e : (e >> 1);
            x[cb] = __uint_as_float(uint32_t(127 + e1) << 23);
            y[cb] = __uint_as_float(uint32_t(127 + e - e1) << 23);
          } else {
            x[cb] = l * r;
          }
        }
      };
      if constexpr(F::scaled) load_group(0, fx, fy);
      bool group_single = true;  // F16: every chunk of the current group has y = 1
      // chunk buffers of chunk c: C under this warp's 32 rows x HALF columns
      // (and their mirror) is prefetched into L2 a few chunks before the
      // tile's end, ahead of the epilogue's loads (prefetching the next
      // tile's C a whole epilogue ahead was slower: 178 -> 190 us at
      // M = N = 8192, K = 64); the chunk's buffer is released on the first
      // CTA's barrier when its columns are in registers
      auto release = [&](int b) {
        umma::fence_before_sync();
        __syncwarp();
        if(lane == 0) {
          if constexpr(F::CG == 2)
            mbar_arrive_cluster(b ? chunk_empty_pair[1] : chunk_empty_pair[0]);
          else
            mbar_arrive(&chunk_empty[b]);
        }
      };
      if constexpr(F::scaled) {
        // chunk c: its factors from lane c % 32, then acc = chunk x factor + acc
        auto consume = [&](int c) -> bool {
          const int b = chunk % F::NBUF;
          if(!F::CEPI && c == max(0, chunks - 4) && beta != 0.f && role != 2) prefetch_c_warp<F>(ti, rank, q, h, lane);
          if(!mbar_wait(&chunk_full[b], (chunk / F::NBUF) & 1, err, kDevErrMmaWait)) return false;
          umma::fence_after_sync();
          const uint32_t base = tmem + (uint32_t(32 * q) << 16) + uint32_t(b) * F::BUF_COLS + uint32_t(h * F::HALF);
          float x[NCB], y[NCB];
          bool single = true;  // every y is 1 (the same in all lanes: one row block, the same column blocks)
#pragma unroll
          for(int cb = 0; cb < NCB; ++cb) {
            x[cb] = __shfl_sync(0xffffffffu, fx[cb], c & 31);
            y[cb] = 1.f;
            if constexpr(F::elem == Elem::F16) {
              if(!group_single) {
                y[cb] = __shfl_sync(0xffffffffu, fy[cb], c & 31);
                single = single && y[cb] == 1.f;
              }
            }
          }
#pragma unroll
          for(int j = 0; j < F::HALF / 32; ++j) {
            uint32_t r[32];
            umma::tmem_ld_32x32b_x32(base + 32 * j, r);
            umma::tmem_ld_wait();
            const int cb = min(32 * j / F::SCALE_ROWS, NCB - 1);
            if(single) {
#pragma unroll
              for(int i = 0; i < 32; ++i)
                acc[32 * j + i] = fmaf(__uint_as_float(r[i]), x[cb], c == 0 ? 0.f : acc[32 * j + i]);
            } else {
#pragma unroll
              for(int i = 0; i < 32; ++i)
                acc[32 * j + i] = fmaf(__uint_as_float(r[i]) * x[cb], y[cb], c == 0 ? 0.f : acc[32 * j + i]);
            }
          }
          release(b);
          return true;
        };
        // groups of 32 chunks, the next group's factors loaded as each
        // group starts (outside the chunk loop, so that they are not
        // predicated into every chunk)
        for(int c0 = 0; c0 < chunks && ok; c0 += 32) {
          if(c0 > 0) {
#pragma unroll
            for(int cb = 0; cb < NCB; ++cb) fx[cb] = nx[cb], fy[cb] = ny[cb];
          }
          if constexpr(F::elem == Elem::F16) {
            // the whole group needs one factor per block (the usual case):
            // its chunks skip the second factor's shuffles
            bool one = true;
#pragma unroll
            for(int cb = 0; cb < NCB; ++cb) one = one && fy[cb] == 1.f;
            group_single = __all_sync(0xffffffffu, one);
          }
          load_group(c0 / 32 + 1, nx, ny);
          for(int c = c0; c < min(chunks, c0 + 32); ++c, ++chunk)
            if(!consume(c)) {
              ok = false;
              break;
            }
        }
      } else {
        for(int c = 0; c < chunks; ++c, ++chunk) {
          const int b = chunk % F::NBUF;
          if(!F::CEPI && c == max(0, chunks - 4) && beta != 0.f && role != 2) prefetch_c_warp<F>(ti, rank, q, h, lane);
          if(!mbar_wait(&chunk_full[b], (chunk / F::NBUF) & 1, err, kDevErrMmaWait)) {
            ok = false;
            break;
          }
          umma::fence_after_sync();
          const uint32_t base = tmem + (uint32_t(32 * q) << 16) + uint32_t(b) * F::BUF_COLS + uint32_t(h * F::HALF);
#pragma unroll
          for(int j = 0; j < F::HALF / 32; ++j) {
            uint32_t r[32];
            umma::tmem_ld_32x32b_x32(base + 32 * j, r);
            umma::tmem_ld_wait();
#pragma unroll
            for(int i = 0; i < 32; ++i) {
              const float v = __uint_as_float(r[i]);
              acc[32 * j + i] = (c == 0) ? v : acc[32 * j + i] + v;
            }
          }
          release(b);
        }
      }
      if(!ok) continue;
      if constexpr(F::CEPI) {
        // C = alpha acc + beta C in the boxes (lane = row: eight 16-byte
        // chunks, swizzled by row, so each quarter warp covers all banks),
        // then TMA stores (clipped at the matrix edges)
        if(beta != 0.f) {
          if(!mbar_wait(&cbar[warp - 4], (c_loads - 1) & 1, err, kDevErrMmaWait)) {
            ok = false;
            continue;
          }
        } else {
          if(lane == 0 && c_stores > 0) bulk_wait_read_all();
          __syncwarp();
        }
#pragma unroll
        for(int j = 0; j < F::HALF / 32; ++j) {
          char* row = cbox + j * F::C_BOX + lane * 128;
#pragma unroll
          for(int k = 0; k < 8; ++k) {
            float4* p4 = reinterpret_cast<float4*>(row + ((k ^ (lane & 7)) << 4));
            const float4 cv = beta != 0.f ? *p4 : make_float4(0.f, 0.f, 0.f, 0.f);
            float4 o;
            o.x = fmaf(beta, cv.x, alpha * acc[32 * j + 4 * k]);
            o.y = fmaf(beta, cv.y, alpha * acc[32 * j + 4 * k + 1]);
            o.z = fmaf(beta, cv.z, alpha * acc[32 * j + 4 * k + 2]);
            o.w = fmaf(beta, cv.w, alpha * acc[32 * j + 4 * k + 3]);
            *p4 = o;
          }
        }
        fence_proxy_async_smem();
        __syncwarp();
        if(lane == 0) {
#pragma unroll
          for(int j = 0; j < F::HALF / 32; ++j) tma_store_2d(&sched.cmap, cbox + j * F::C_BOX, nbase + 32 * j, crow);
          bulk_commit();
        }
        ++c_stores;
        continue;
      }
      // K-split tile: the second half stores its sums (partial tile of the
      // CTA: 128 rows x BN, row-major), the first half waits for them and
      // adds them to its own (first + second) before writing C
      float* part = nullptr;
      if(F::CG == 2 && role != 0) {
        part = sched.partial + ((size_t(slot) * F::CG + rank) * 128 + 32 * q) * F::BN + h * F::HALF + lane;
        if(role == 1 && !wait_count(&sched.flags[slot], 8 * F::CG, err, kDevErrSplitWait)) {
          ok = false;
          continue;
        }
      }
      // Write C through a per-warp 32 x 32 staging tile: each lane holds one
      // row of the block, the stores go out one 128-byte row segment per
      // instruction (coalesced for any ldc and alignment).
      float(*stage)[33] = epi_stage + (warp - 4) * 32;
      const int row0 = ti.m0 + int(rank) * F::BM_CTA + 32 * q;
#pragma unroll
      for(int j = 0; j < F::HALF / 32; ++j) {
#pragma unroll
        for(int i = 0; i < 32; ++i) stage[lane][i] = acc[32 * j + i];
        __syncwarp();
        if(F::CG == 2 && role != 0) {
          float* pj = part + 32 * j;  // column lane of this warp's 32 rows
          if(role == 2) {
#pragma unroll 4
            for(int r = 0; r < 32; ++r) __stcg(pj + r * F::BN, stage[r][lane]);
            __syncwarp();
            continue;
          }
#pragma unroll 4
          for(int r = 0; r < 32; ++r) stage[r][lane] += __ldcg(pj + r * F::BN);
          __syncwarp();
        }
        const int n = nbase + 32 * j + lane;
        if(n < N) {
          const int rows = min(32, M - row0);
          float* col = ti.C + int64_t(row0) * ldc + n;
          // a batch of loads in flight before its first store (16 while 128
          // accumulator columns per warp are still live)
          constexpr int kBatch = F::HALF > 64 ? 16 : 32;
#pragma unroll
          for(int r0 = 0; r0 < 32; r0 += kBatch) {
            float cv[kBatch];
#pragma unroll
            for(int r = 0; r < kBatch; ++r)
              cv[r] = (beta != 0.f && r0 + r < rows) ? col[int64_t(r0 + r) * ldc] : 0.f;
#pragma unroll
            for(int r = 0; r < kBatch; ++r)
              if(r0 + r < rows) col[int64_t(r0 + r) * ldc] = fmaf(beta, cv[r], alpha * stage[r0 + r][lane]);
          }
        }
        if constexpr(F::MIRROR) {
          if(ti.mirror) {
          // transpose: C[n0 + 32j + r][row0 + lane] from the product element (row0 + lane, n0 + 32j + r)
          const int mrow0 = nbase + 32 * j, mcol = row0 + lane;
          if(mcol < M) {
            const int rows = min(32, N - mrow0);
            float* col = ti.C + int64_t(mrow0) * ldc + mcol;
            constexpr int kMBatch = F::HALF > 64 ? 8 : 16;  // loads in flight at a time
#pragma unroll
            for(int half = 0; half < 32; half += kMBatch) {
              float cv[kMBatch];
#pragma unroll
              for(int r = 0; r < kMBatch; ++r)
                cv[r] = (beta != 0.f && half + r < rows) ? col[int64_t(half + r) * ldc] : 0.f;
#pragma unroll
              for(int r = 0; r < kMBatch; ++r)
                if(half + r < rows) col[int64_t(half + r) * ldc] = fmaf(beta, cv[r], alpha * stage[lane][half + r]);
            }
          }
          }
        }
        __syncwarp();
      }
      if(F::CG == 2 && role == 2) {  // sums stored: count this warp
        __threadfence();
        __syncwarp();
        if(lane == 0) atomicAdd(&sched.flags[slot], 1);
      }
    }
    if constexpr(F::CEPI)
      if(lane == 0 && c_stores > 0) bulk_wait_all();  // C written before the CTA leaves
  }

  umma::fence_before_sync();
  if constexpr(F::CG == 2) {
    // neither CTA leaves (or frees TMEM) while the pair's MMAs, copies or
    // barrier arrivals may still target it
    cluster_sync();
    if(warp == 1) {
      umma::fence_after_sync();
      umma::tmem_dealloc_pair(tmem, F::TMEM_COLS);
    }
  } else {
    __syncthreads();
    if(warp == 1) {
      umma::fence_after_sync();
      umma::tmem_dealloc(tmem, F::TMEM_COLS);
    }
  }
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Panels {
  char* base;     // term 0
  size_t stride;  // bytes between terms
};

template <class F>
gbpoly_status launch_split(gbpoly_ctx* ctx, const float* X, int64_t ld, bool k_major, int64_t rows, int64_t K,
    int64_t Kp, Panels out, RowXform xf = RowXform{}, float* inv_scale = nullptr) {
  using T = typename Term<F::elem>::T;
  dim3 grid(static_cast<unsigned>(Kp / 64), static_cast<unsigned>((rows + 63) / 64));
  if(grid.y > 65535u) return fail(GBPOLY_ERR_UNSUPPORTED, "operand too large for the split pass (over 65535 row blocks)");
  ProfileScope prof(ctx, "split_terms");
  split_kernel<F::elem, F::terms><<<grid, 256, 0, ctx->stream>>>(X, ld, k_major ? 1 : 0, int(rows), int(K), int(Kp),
      reinterpret_cast<T*>(out.base), int64_t(out.stride / sizeof(T)), xf, inv_scale);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

template <class F>
gbpoly_status make_product_maps(gbpoly_ctx* ctx, ProductMaps& pm, Panels left, int64_t left_rows, Panels right,
    int64_t right_rows, int64_t Kp) {
  const auto dt = F::elem == Elem::BF16   ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                  : F::elem == Elem::F16  ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                  : F::elem == Elem::TF32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                          : CU_TENSOR_MAP_DATA_TYPE_UINT8;
  const auto sw = F::ROW == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
  gbpoly_status st;
  for(int t = 0; t < F::terms; ++t) {
    if((st = make_tmap_2d(ctx, &pm.l[t], dt, F::esz, left.base + t * left.stride, left_rows, Kp, Kp, F::BM_CTA,
            F::BK, sw)) != GBPOLY_OK)
      return st;
    if((st = make_tmap_2d(ctx, &pm.r[t], dt, F::esz, right.base + t * right.stride, right_rows, Kp, Kp, F::BN_CTA,
            F::BK, sw)) != GBPOLY_OK)
      return st;
  }
  return GBPOLY_OK;
}

// Once per device context: shared-memory opt-in and the register check of
// the warp split.
template <class F, class S>
gbpoly_status tc_prepare(gbpoly_ctx* ctx) {
  static ContextMark prepared;
  if(prepared.valid(ctx->device)) return GBPOLY_OK;
  GBPOLY_CUDA_TRY(cudaFuncSetAttribute(split_gemm_kernel<F, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, F::SMEM));
  // setmaxnreg redistributes the registers the CTA was launched with: the
  // split must fit in threads x registers-per-thread at launch, or the
  // increase would wait forever.
  cudaFuncAttributes fa;
  GBPOLY_CUDA_TRY(cudaFuncGetAttributes(&fa, split_gemm_kernel<F, S>));
  const long need = 128l * F::REGS_CTRL + 256l * F::REGS_EPI;
  if(long(fa.numRegs) * F::THREADS < need)
    return fail(GBPOLY_ERR_UNSUPPORTED, "tensor-core kernel built with too few registers for its warp split");
  prepared.set(ctx->device);
  return GBPOLY_OK;
}

// Launch configuration of a CTA-pair kernel: clusters of two along x.
template <class F>
struct PairLaunch {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  PairLaunch(gbpoly_ctx* ctx, int clusters) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(2 * clusters);
    cfg.blockDim = dim3(F::THREADS);
    cfg.dynamicSmemBytes = F::SMEM;
    cfg.stream = ctx->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
};

// CTA pairs of configuration F resident at once on the device (cached per
// device context).
template <class F, class S>
gbpoly_status pair_clusters(gbpoly_ctx* ctx, int& clusters) {
  static int max_clusters[32] = {};
  static ContextMark known;
  gbpoly_status st = tc_prepare<F, S>(ctx);
  if(st != GBPOLY_OK) return st;
  if(known.valid(ctx->device)) {
    clusters = max_clusters[ctx->device];
    return GBPOLY_OK;
  }
  PairLaunch<F> pl(ctx, ctx->sm_count / 2);
  int n = 0;
  GBPOLY_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n, split_gemm_kernel<F, S>, &pl.cfg));
  if(n <= 0) return fail(GBPOLY_ERR_UNSUPPORTED, "no CTA pair of this tensor-core configuration fits on the device");
  if(ctx->device >= 0 && ctx->device < 32) {
    max_clusters[ctx->device] = n;
    known.set(ctx->device);
  }
  clusters = n;
  return GBPOLY_OK;
}

// K-split tail of a CTA-pair launch.  When the last round of tiles would
// leave half the resident pairs or more idle, each of its `slots` tiles runs
// as two units of half the K chunks; `bytes` of workspace hold their partial
// sums and arrival counters.  Only launches of fewer than kTailMaxRounds
// full rounds split: with more, the last round is a small share of the time
// and pairing two clusters on one tile (the first half waits for the second)
// costs about what it saves (measured on GB300: +6 to +15% at 2560 and 4096,
// -1 to -3% at 8192).
struct TailPlan {
  int64_t units = 0;  // work units of the launch
  int full_tiles = 0, split_it = 0, slots = 0;
  size_t bytes = 0;
};
constexpr size_t kTailSlotBytes = size_t(256) * 256 * sizeof(float);  // one 256 x 256 FP32 tile
constexpr int kTailMaxRounds = 8;

template <class F, class S>
gbpoly_status plan_tail(gbpoly_ctx* ctx, int64_t tiles, int64_t iters, TailPlan& tp) {
  tp = TailPlan{};
  tp.units = tiles;
  if constexpr(F::CG == 2 && !F::CEPI) {
    static_assert(size_t(F::BM) * F::BN * sizeof(float) == kTailSlotBytes, "tail slot size");
    const int64_t chunks = (iters + F::CH - 1) / F::CH;
    if(!ctx->tail_split || tiles <= 0 || chunks < 2) return GBPOLY_OK;
    int P = 0;
    gbpoly_status st = pair_clusters<F, S>(ctx, P);
    if(st != GBPOLY_OK) return st;
    const int64_t R = tiles % P;
    if(R > 0 && 2 * R <= P && tiles / P < kTailMaxRounds) {
      tp.full_tiles = int(tiles - R);
      tp.units = tiles + R;
      tp.split_it = int(chunks / 2 * F::CH);
      tp.slots = int(R);
      tp.bytes = size_t(R) * kTailSlotBytes + align_up(size_t(R) * sizeof(int), 256);
    }
  }
  return GBPOLY_OK;
}

// Point the scheduler at the tail's workspace (at `base`) and clear its counters.
template <class S>
gbpoly_status apply_tail(gbpoly_ctx* ctx, const TailPlan& tp, char* base, S& sched) {
  if(tp.slots == 0) return GBPOLY_OK;
  sched.units = int(tp.units);
  sched.full_tiles = tp.full_tiles;
  sched.split_it = tp.split_it;
  sched.partial = reinterpret_cast<float*>(base);
  sched.flags = reinterpret_cast<int*>(base + size_t(tp.slots) * kTailSlotBytes);
  GBPOLY_CUDA_TRY(cudaMemsetAsync(sched.flags, 0, size_t(tp.slots) * sizeof(int), ctx->stream));
  return GBPOLY_OK;
}

// Launch the tensor-core kernel for scheduler S: one persistent CTA (or CTA
// pair) per SM (pair of SMs), walking `units` work units.
template <class F, class S>
gbpoly_status launch_tc_kernel(gbpoly_ctx* ctx, const S& sched, int64_t units, const char* kernel_name) {
  gbpoly_status st = tc_prepare<F, S>(ctx);
  if(st != GBPOLY_OK) return st;
  if(units <= 0) return GBPOLY_OK;
  if constexpr(F::CG == 2) {
    // CTA pairs: a cluster of two per tile, as many clusters as fit at once
    int P = 0;
    if((st = pair_clusters<F, S>(ctx, P)) != GBPOLY_OK) return st;
    PairLaunch<F> pl(ctx, int(std::min<int64_t>(units, P)));
    ProfileScope prof(ctx, kernel_name);
    GBPOLY_CUDA_TRY(cudaLaunchKernelEx(&pl.cfg, split_gemm_kernel<F, S>, sched, ctx->err_dev));
    return GBPOLY_OK;
  }
  const int grid = int(std::min<int64_t>(units, ctx->sm_count));
  ProfileScope prof(ctx, kernel_name);
  split_gemm_kernel<F, S><<<grid, F::THREADS, F::SMEM, ctx->stream>>>(sched, ctx->err_dev);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

// Workspace layout: terms x [A panel] then terms x [B panel] (B absent when
// both operands are the same rows).
struct Layout {
  int64_t Kp;
  size_t a_stride, b_stride, a_bytes, b_bytes;
};

template <class F>
Layout layout(int64_t M, int64_t N, int64_t K, bool same) {
  Layout l;
  l.Kp = align_up(size_t(std::max<int64_t>(K, 1)), 64);
  l.a_stride = align_up(size_t(M) * l.Kp * F::esz, 1024);
  l.b_stride = align_up(size_t(N) * l.Kp * F::esz, 1024);
  l.a_bytes = F::terms * l.a_stride;
  l.b_bytes = same ? 0 : F::terms * l.b_stride;
  return l;
}

// syrk: both operands are the rows of A; split once
bool same_operand(const GemmF32Args& a) { return symmetric_operand(a); }

// C rows that TMA can load and store: 16-byte-aligned base and row pitch, and
// rows ending on a 16-byte boundary (TMA stores clip the row end at 16-byte
// granularity: a ragged N would write into the padding of ldc).
bool c_tile_ok(const GemmF32Args& a) {
  return (reinterpret_cast<uintptr_t>(a.C) & 15) == 0 && (a.ldc & 3) == 0 && (a.N & 3) == 0;
}

template <class F>
gbpoly_status run_form(gbpoly_ctx* ctx, const GemmF32Args& a, const char* kernel_name) {
  if(a.M == 0 || a.N == 0) return GBPOLY_OK;
  if(a.M >= (1ll << 31) || a.N >= (1ll << 31) || a.K >= (1ll << 30))
    return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large for the tensor-core kernels");
  const bool same = same_operand(a);
  if(a.xf.mean && !same) return fail(GBPOLY_ERR_UNSUPPORTED, "row transform: symmetric products only");
  const Layout lay = layout<F>(a.M, a.N, a.K, same);
  const int64_t Kp = lay.Kp;
  const size_t a_stride = lay.a_stride, b_stride = lay.b_stride, a_bytes = lay.a_bytes, b_bytes = lay.b_bytes;
  using Sched = SingleSched<F::BM, F::BN>;
  int64_t tiles = ((a.M + F::BM - 1) / F::BM) * ((a.N + F::BN - 1) / F::BN);
  const bool lower = F::MIRROR && (same || a.dual) && a.M == a.N;  // symmetric product: lower triangle of tiles
  if(lower) {
    const int64_t t = (a.M + F::BM - 1) / F::BM;
    tiles = t * (t + 1) / 2;
  }
  TailPlan tail;
  gbpoly_status st = plan_tail<F, Sched>(ctx, tiles, (Kp / F::BK) * (a.dual ? 2 : 1), tail);
  if(st != GBPOLY_OK) return st;
  // F16 terms: inverse block scales after the panels, [64-row block][64-K block]
  const int64_t kt = Kp / 64;
  const size_t sa_bytes = F::elem == Elem::F16 ? align_up(size_t((a.M + 63) / 64) * size_t(kt) * 4, 256) : 0;
  const size_t sb_bytes = F::elem == Elem::F16 && !same ? align_up(size_t((a.N + 63) / 64) * size_t(kt) * 4, 256) : 0;
  if((st = ensure_workspace(ctx, a_bytes + b_bytes + sa_bytes + sb_bytes + tail.bytes)) != GBPOLY_OK) return st;
  char* ws = static_cast<char*>(ctx->ws.ptr);
  Panels pa{ws, a_stride};
  Panels pb = same ? pa : Panels{ws + a_bytes, b_stride};
  float* const sa = F::elem == Elem::F16 ? reinterpret_cast<float*>(ws + a_bytes + b_bytes) : nullptr;
  float* const sb = same ? sa : (F::elem == Elem::F16 ? reinterpret_cast<float*>(ws + a_bytes + b_bytes + sa_bytes) : nullptr);
  if(a.K > 0 || F::elem == Elem::F16) {  // (F16: the split also writes the scales; with K = 0 they are 1)
    if((st = launch_split<F>(ctx, a.A, a.lda, a.op_a == GBPOLY_OP_N, a.M, a.K, Kp, pa, a.xf, sa)) != GBPOLY_OK)
      return st;
    if(!same && (st = launch_split<F>(ctx, a.B, a.ldb, a.op_b == GBPOLY_OP_T, a.N, a.K, Kp, pb, RowXform{}, sb)) !=
                    GBPOLY_OK)
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

  Sched sched{maps, npair, int(a.M), int(a.N), int(Kp), a.alpha, a.beta, a.C, a.ldc};
  sched.lower = lower;
  if constexpr(F::elem == Elem::F16) {
    sched.sl[0] = sa, sched.sr[0] = sb;
    sched.sl[1] = sb, sched.sr[1] = sa;  // syr2k's second pairing, B_i . A_j^T
    sched.kt = int(kt);
  }
  if constexpr(F::CEPI) {
    if(lower || !c_tile_ok(a)) return fail(GBPOLY_ERR_UNSUPPORTED, "C-tile epilogue: non-symmetric, 16-byte-aligned C");
    if((st = make_tmap_2d(ctx, &sched.cmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, a.C, a.M, a.N, a.ldc, 32, 32,
            CU_TENSOR_MAP_SWIZZLE_128B)) != GBPOLY_OK)
      return st;
  }
  if((st = apply_tail(ctx, tail, ws + a_bytes + b_bytes + sa_bytes + sb_bytes, sched)) != GBPOLY_OK) return st;
  return launch_tc_kernel<F>(ctx, sched, tail.units, kernel_name);
}

// FP8 form: quantize both operands (panels + block scales), one MMA product.
template <class F>
gbpoly_status run_fp8(gbpoly_ctx* ctx, const GemmF32Args& a) {
  if(a.xf.mean) return fail(GBPOLY_ERR_UNSUPPORTED, "row transform: split forms only");
  if(a.M == 0 || a.N == 0) return GBPOLY_OK;
  if(a.M >= (1ll << 31) || a.N >= (1ll << 31) || a.K >= (1ll << 30))
    return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large for the tensor-core kernels");
  const bool same = same_operand(a);
  const int64_t Kp = int64_t(align_up(size_t(std::max<int64_t>(a.K, 1)), 128));
  const int64_t mb = (a.M + 127) / 128, nb = (a.N + 127) / 128, kb = Kp / 128;
  const size_t a_bytes = align_up(size_t(a.M) * Kp, 1024), b_bytes = same ? 0 : align_up(size_t(a.N) * Kp, 1024);
  const size_t sa_bytes = align_up(size_t(mb * kb) * 4, 256), sb_bytes = same ? 0 : align_up(size_t(nb * kb) * 4, 256);
  gbpoly_status st = ensure_workspace(ctx, a_bytes + b_bytes + sa_bytes + sb_bytes);
  if(st != GBPOLY_OK) return st;
  char* ws = static_cast<char*>(ctx->ws.ptr);
  uint8_t* qa = reinterpret_cast<uint8_t*>(ws);
  uint8_t* qb = same ? qa : reinterpret_cast<uint8_t*>(ws + a_bytes);
  float* sa = reinterpret_cast<float*>(ws + a_bytes + b_bytes);
  float* sb = same ? sa : reinterpret_cast<float*>(ws + a_bytes + b_bytes + sa_bytes);
  {
    ProfileScope prof(ctx, "quantize_e4m3");
    const QuantJob ja{a.A, a.lda, a.op_a == GBPOLY_OP_N ? 1 : 0, int(a.M), int(a.K), int(Kp), int(kb), qa, sa};
    const QuantJob jb{a.B, a.ldb, a.op_b == GBPOLY_OP_T ? 1 : 0, int(a.N), int(a.K), int(Kp), int(kb), qb, sb};
    const int64_t blocks_a = mb * kb, blocks = blocks_a + (same ? 0 : nb * kb);
    if(blocks >= (1ll << 31)) return fail(GBPOLY_ERR_UNSUPPORTED, "too many quantisation blocks");
    // persistent: two CTAs per SM walk the blocks (no launch and drain per block)
    const unsigned ctas = unsigned(std::min<int64_t>(blocks, 2 * int64_t(std::max(1, ctx->sm_count))));
    quantize_e4m3_kernel<<<ctas, 512, 0, ctx->stream>>>(ja, jb, int(blocks_a), int(blocks));
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  GemmMaps maps;
  int npair = 1;
  Panels pa{reinterpret_cast<char*>(qa), a_bytes}, pb{reinterpret_cast<char*>(qb), b_bytes};
  if((st = make_product_maps<F>(ctx, maps.p[0], pa, a.M, pb, a.N, Kp)) != GBPOLY_OK) return st;
  SingleSched<F::BM, F::BN> sched{maps, npair, int(a.M), int(a.N), int(Kp), a.alpha, a.beta, a.C, a.ldc};
  sched.sl[0] = sa;
  sched.sr[0] = sb;
  sched.kt = int(kb);
  if(a.dual) {  // syr2k: B_i . A_j^T
    sched.npair = 2;
    if((st = make_product_maps<F>(ctx, sched.maps.p[1], pb, a.M, pa, a.N, Kp)) != GBPOLY_OK) return st;
    sched.sl[1] = sb;
    sched.sr[1] = sa;
  } else {
    sched.maps.p[1] = sched.maps.p[0];
  }
  const int64_t tiles = ((a.M + F::BM - 1) / F::BM) * ((a.N + F::BN - 1) / F::BN);
  return launch_tc_kernel<F>(ctx, sched, tiles, "fp8_gemm");
}

template <class F>
size_t bytes_of(int64_t M, int64_t N, int64_t K, bool same) {
  const Layout l = layout<F>(M, N, K, same);
  return l.a_bytes + l.b_bytes;
}

}  // namespace

size_t workspace_bytes(gbpoly_precision prec, int64_t M, int64_t N, int64_t K, bool same) {
  // The largest over the configurations of the form (they differ only in
  // padding), plus the K-split tail of CTA-pair configurations: at most half
  // the resident pairs of a device of up to 256 SMs, and no more than the
  // shape's 256 x 256 tiles.
  const int64_t slots = std::min<int64_t>(64, ((M + 255) / 256) * ((N + 255) / 256));
  const size_t tail = size_t(slots) * kTailSlotBytes + align_up(size_t(slots) * sizeof(int), 256);
  switch(prec) {
  case GBPOLY_PREC_TF32: return bytes_of<FormTF32>(M, N, K, same) + tail;
  case GBPOLY_PREC_BF16X3: return bytes_of<FormBF16x3>(M, N, K, same) + tail;
  case GBPOLY_PREC_TF32X3: return bytes_of<FormTF32x3>(M, N, K, same) + tail;
  case GBPOLY_PREC_BF16X6: return bytes_of<FormBF16x6>(M, N, K, same) + tail;
  case GBPOLY_PREC_FP16X3: {
    const size_t kt = align_up(size_t(std::max<int64_t>(K, 1)), 64) / 64;
    return bytes_of<FormF16x3>(M, N, K, same) + tail + align_up(size_t((M + 63) / 64) * kt * 4, 256) +
           (same ? 0 : align_up(size_t((N + 63) / 64) * kt * 4, 256));
  }
  case GBPOLY_PREC_FP8: {
    const size_t Kp = align_up(size_t(std::max<int64_t>(K, 1)), 128), kb = Kp / 128;
    return align_up(size_t(M) * Kp, 1024) + (same ? 0 : align_up(size_t(N) * Kp, 1024)) +
           align_up(size_t((M + 127) / 128) * kb * 4, 256) + (same ? 0 : align_up(size_t((N + 127) / 128) * kb * 4, 256));
  }
  case GBPOLY_PREC_FP32:
    // partial products of the K split of small grids, bounded for devices of up to 256 SMs
    return fp32_split_k_bytes(256, M, N, K);
  default: return 0;
  }
}

int tensor_config_count(gbpoly_precision prec) {
  switch(prec) {
  case GBPOLY_PREC_TF32:
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_TF32X3:
  case GBPOLY_PREC_BF16X6: return 6;  // configurations 3, 4, 5: CTA pairs (5: C tile in shared memory)
  case GBPOLY_PREC_FP8: return 2;  // configuration 1: 128 x 256 tiles
  case GBPOLY_PREC_FP16X3: return 3;  // 0: 128 x 256, 1: 128 x 128, 2: CTA pairs 256 x 256
  default: return 0;
  }
}

gbpoly_status launch_gemm_tensor_config(gbpoly_ctx* ctx, gbpoly_precision prec, int config, const GemmF32Args& a) {
  switch(prec * 8 + config) {
  case GBPOLY_PREC_TF32 * 8 + 0: return run_form<FormTF32>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 1: return run_form<FormTF32_b>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 2: return run_form<FormTF32_c>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 3: return run_form<FormTF32_p>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 4: return run_form<FormTF32_q>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 5: return run_form<FormTF32_t>(ctx, a, "tf32_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 0: return run_form<FormBF16x3>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 1: return run_form<FormBF16x3_b>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 2: return run_form<FormBF16x3_c>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 3: return run_form<FormBF16x3_p>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 4: return run_form<FormBF16x3_q>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 5: return run_form<FormBF16x3_t>(ctx, a, "bf16x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 0: return run_form<FormTF32x3>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 1: return run_form<FormTF32x3_b>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 2: return run_form<FormTF32x3_c>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 3: return run_form<FormTF32x3_p>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 4: return run_form<FormTF32x3_q>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 5: return run_form<FormTF32x3_t>(ctx, a, "tf32x3_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 0: return run_form<FormBF16x6>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 1: return run_form<FormBF16x6_b>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 2: return run_form<FormBF16x6_c>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 3: return run_form<FormBF16x6_p>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 4: return run_form<FormBF16x6_q>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 5: return run_form<FormBF16x6_t>(ctx, a, "bf16x6_gemm");
  case GBPOLY_PREC_FP8 * 8 + 0: return run_fp8<FormFP8>(ctx, a);
  case GBPOLY_PREC_FP8 * 8 + 1: return run_fp8<FormFP8_w>(ctx, a);
  case GBPOLY_PREC_FP16X3 * 8 + 0: return run_form<FormF16x3>(ctx, a, "fp16x3_gemm");
  case GBPOLY_PREC_FP16X3 * 8 + 1: return run_form<FormF16x3_c>(ctx, a, "fp16x3_gemm");
  case GBPOLY_PREC_FP16X3 * 8 + 2: return run_form<FormF16x3_p>(ctx, a, "fp16x3_gemm");
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision form or tile configuration not available");
  }
}

// -------------------------------------------------- panel-wise contraction
// One row panel [r0, r0 + a.M) of a contraction whose full A has Mfull rows:
// the workspace holds the term panels of all of A (rows r0.. of this call)
// followed by those of B, which the first panel splits once.
template <class F>
gbpoly_status run_form_panel(gbpoly_ctx* ctx, const GemmF32Args& a, int64_t Mfull, bool first, int64_t r0,
    const char* name) {
  const Layout lay = layout<F>(Mfull, a.N, a.K, false);
  gbpoly_status st = ensure_workspace(ctx, lay.a_bytes + lay.b_bytes);
  if(st != GBPOLY_OK) return st;
  char* ws = static_cast<char*>(ctx->ws.ptr);
  Panels pa{ws + size_t(r0) * lay.Kp * F::esz, lay.a_stride};
  Panels pb{ws + lay.a_bytes, lay.b_stride};
  if(first && (st = launch_split<F>(ctx, a.B, a.ldb, a.op_b == GBPOLY_OP_T, a.N, a.K, lay.Kp, pb)) != GBPOLY_OK)
    return st;
  if((st = launch_split<F>(ctx, a.A, a.lda, a.op_a == GBPOLY_OP_N, a.M, a.K, lay.Kp, pa)) != GBPOLY_OK) return st;
  GemmMaps maps;
  if((st = make_product_maps<F>(ctx, maps.p[0], pa, a.M, pb, a.N, lay.Kp)) != GBPOLY_OK) return st;
  maps.p[1] = maps.p[0];
  SingleSched<F::BM, F::BN> sched{maps, 1, int(a.M), int(a.N), int(lay.Kp), a.alpha, a.beta, a.C, a.ldc};
  const int64_t tiles = ((a.M + F::BM - 1) / F::BM) * ((a.N + F::BN - 1) / F::BN);
  return launch_tc_kernel<F>(ctx, sched, tiles, name);
}

// Square-tile configurations of each form (128 x 128, or 256 x 256 for CTA
// pairs): symmetric updates need one to compute only the lower triangle of
// tiles.
namespace {
bool config_is_square(gbpoly_precision prec, int config) {
  switch(prec) {
  case GBPOLY_PREC_TF32:
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_TF32X3: return config == 2 || config == 3 || config == 4;
  case GBPOLY_PREC_BF16X6: return config == 0 || config == 1 || config == 3 || config == 4;
  case GBPOLY_PREC_FP8: return config == 0;
  case GBPOLY_PREC_FP16X3: return config == 1 || config == 2;
  default: return false;
  }
}
// CTA pairs when their 256 x 256 tiles give every SM pair at least one tile.
bool pairs_fill(gbpoly_ctx* ctx, int64_t pair_tiles) { return pair_tiles >= std::max(1, ctx->sm_count / 2); }
int square_config(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t N) {
  if(prec == GBPOLY_PREC_FP8) return 0;
  const int64_t t = (N + 255) / 256;
  if(prec == GBPOLY_PREC_FP16X3) return pairs_fill(ctx, t * (t + 1) / 2) ? 2 : 1;
  if(pairs_fill(ctx, t * (t + 1) / 2)) return 3;
  return prec == GBPOLY_PREC_BF16X6 ? 1 : 2;
}
}  // namespace

// Configuration of an untuned shape: CTA pairs (256 x 256 tiles) when they
// fill the device, with the C tile in shared memory (configuration 5) while
// K is short enough that C's traffic bounds the call (measured on GB300 at
// M = N = 8192: 1.75x faster up to K = 128, ahead up to K = 256 for the
// BF16 forms and K = 512 for tf32, behind beyond), else the 1-CTA
// configuration with the most tiles.
int default_config(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K) {
  // fp8: 128 x 256 tiles (twice the MMA work per scaled chunk: 1.38x at
  // N = 8192) when they give every SM a tile, else 128 x 128
  if(prec == GBPOLY_PREC_FP8) return ((M + 127) / 128) * ((N + 255) / 256) >= ctx->sm_count ? 1 : 0;
  // fp16x3: CTA pairs when they fill the device, else 128 x 128 tiles
  if(prec == GBPOLY_PREC_FP16X3) return pairs_fill(ctx, ((M + 255) / 256) * ((N + 255) / 256)) ? 2 : 1;
  if(tensor_config_count(prec) <= 3) return 0;
  if(pairs_fill(ctx, ((M + 255) / 256) * ((N + 255) / 256))) {
    const int64_t k_tile = prec == GBPOLY_PREC_TF32 ? 512 : (prec == GBPOLY_PREC_TF32X3 ? 128 : 256);
    return K <= k_tile ? 5 : 3;
  }
  // 128 x 128 tiles: configuration 2 (0 for bf16x6, whose configuration 0 is 128 x 128)
  return prec == GBPOLY_PREC_BF16X6 ? 0 : 2;
}

gbpoly_status tensor_plan(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op, gbpoly_op, int64_t M, int64_t N,
    int64_t K, TensorPlan* plan) {
  if(tensor_config_count(prec) == 0) return fail(GBPOLY_ERR_UNSUPPORTED, "precision form not available");
  plan->prec = prec;
  plan->config = tuned_config(ctx, prec, M, N, K);
  plan->M = M;
  return GBPOLY_OK;
}

gbpoly_status tensor_plan_panel(gbpoly_ctx* ctx, const TensorPlan& plan, const GemmF32Args& a, bool first, int64_t r0) {
  switch(plan.prec * 8 + plan.config) {
  case GBPOLY_PREC_TF32 * 8 + 0: return run_form_panel<FormTF32>(ctx, a, plan.M, first, r0, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 1: return run_form_panel<FormTF32_b>(ctx, a, plan.M, first, r0, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 2: return run_form_panel<FormTF32_c>(ctx, a, plan.M, first, r0, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 3:
  case GBPOLY_PREC_TF32 * 8 + 5: return run_form_panel<FormTF32_p>(ctx, a, plan.M, first, r0, "tf32_gemm");
  case GBPOLY_PREC_TF32 * 8 + 4: return run_form_panel<FormTF32_q>(ctx, a, plan.M, first, r0, "tf32_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 0: return run_form_panel<FormBF16x3>(ctx, a, plan.M, first, r0, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 1: return run_form_panel<FormBF16x3_b>(ctx, a, plan.M, first, r0, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 2: return run_form_panel<FormBF16x3_c>(ctx, a, plan.M, first, r0, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 3:
  case GBPOLY_PREC_BF16X3 * 8 + 5: return run_form_panel<FormBF16x3_p>(ctx, a, plan.M, first, r0, "bf16x3_gemm");
  case GBPOLY_PREC_BF16X3 * 8 + 4: return run_form_panel<FormBF16x3_q>(ctx, a, plan.M, first, r0, "bf16x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 0: return run_form_panel<FormTF32x3>(ctx, a, plan.M, first, r0, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 1: return run_form_panel<FormTF32x3_b>(ctx, a, plan.M, first, r0, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 2: return run_form_panel<FormTF32x3_c>(ctx, a, plan.M, first, r0, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 3:
  case GBPOLY_PREC_TF32X3 * 8 + 5: return run_form_panel<FormTF32x3_p>(ctx, a, plan.M, first, r0, "tf32x3_gemm");
  case GBPOLY_PREC_TF32X3 * 8 + 4: return run_form_panel<FormTF32x3_q>(ctx, a, plan.M, first, r0, "tf32x3_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 0: return run_form_panel<FormBF16x6>(ctx, a, plan.M, first, r0, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 1: return run_form_panel<FormBF16x6_b>(ctx, a, plan.M, first, r0, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 2: return run_form_panel<FormBF16x6_c>(ctx, a, plan.M, first, r0, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 3:
  case GBPOLY_PREC_BF16X6 * 8 + 5: return run_form_panel<FormBF16x6_p>(ctx, a, plan.M, first, r0, "bf16x6_gemm");
  case GBPOLY_PREC_BF16X6 * 8 + 4: return run_form_panel<FormBF16x6_q>(ctx, a, plan.M, first, r0, "bf16x6_gemm");
  case GBPOLY_PREC_FP8 * 8 + 0: return run_fp8<FormFP8>(ctx, a);  // quantises both operands per panel
  case GBPOLY_PREC_FP8 * 8 + 1: return run_fp8<FormFP8_w>(ctx, a);
  // fp16x3: split both operands (and their block scales) per panel
  case GBPOLY_PREC_FP16X3 * 8 + 0: return run_form<FormF16x3>(ctx, a, "fp16x3_gemm");
  case GBPOLY_PREC_FP16X3 * 8 + 1: return run_form<FormF16x3_c>(ctx, a, "fp16x3_gemm");
  case GBPOLY_PREC_FP16X3 * 8 + 2: return run_form<FormF16x3_p>(ctx, a, "fp16x3_gemm");
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision form or tile configuration not available");
  }
}

gbpoly_status launch_gemm_tensor(gbpoly_ctx* ctx, gbpoly_precision prec, const GemmF32Args& a) {
  int config = tuned_config(ctx, prec, a.M, a.N, a.K);
  const bool symmetric = (same_operand(a) || a.dual) && a.M == a.N;
  if(symmetric && !config_is_square(prec, config)) config = square_config(ctx, prec, a.N);
  if(config == 5 && !c_tile_ok(a)) config = 3;  // C rows TMA cannot address: the staged epilogue
  return launch_gemm_tensor_config(ctx, prec, config, a);
}

// ----------------------------------------------------------- grouped calls
//
// Many independent contractions of uneven shapes in two launches: one split
// pass over all operands and one persistent tensor-core launch over the
// tiles of all problems.  A plan prepares everything on the host once (term
// panels, problem table, per-problem tensor maps, the tile list ordered by
// decreasing K so that the round-robin walk of the persistent CTAs balances,
// split jobs) and owns the device memory, so running it only enqueues the
// two kernels and can be captured into a CUDA graph.

}  // namespace gbpoly

struct gbpoly_grouped {
  gbpoly_precision prec;
  std::vector<gbpoly_gemm_desc> descs;  // fp32: run as per-problem launches
  void* dev = nullptr;                  // panels + tables
  size_t dev_bytes = 0;
  gbpoly::GroupProblem* probs = nullptr;
  gbpoly::ProductMaps* maps = nullptr;
  int4* tiles = nullptr;
  gbpoly::SplitJob* jobs = nullptr;
  int4* split_table = nullptr;  // split block -> (job, row block, k block, 0)
  int ntiles = 0, njobs = 0, split_blocks = 0;
  int64_t flops = 0;
  int config = 0;  // tile configuration: 0 128 x 128, 1 CTA pairs 256 x 256, 2 (bf16x3, fp16x3) 128 x 256
};

namespace gbpoly {
namespace {

template <class F>
gbpoly_status plan_grouped(gbpoly_ctx* ctx, gbpoly_grouped* g) {
  const int P = int(g->descs.size());
  // layout: panels first, then problem table, tensor maps, tiles, jobs
  std::vector<size_t> a_off(P), b_off(P);
  std::vector<int64_t> kp(P);
  size_t off = 0;
  for(int i = 0; i < P; ++i) {
    const auto& d = g->descs[i];
    kp[i] = int64_t(align_up(size_t(std::max<int64_t>(d.K, 1)), 64));
    a_off[i] = off;
    off += F::terms * align_up(size_t(d.M) * kp[i] * F::esz, 1024);
    b_off[i] = off;
    off += F::terms * align_up(size_t(d.N) * kp[i] * F::esz, 1024);
  }
  // F16 terms: each operand's inverse block scales after the panels
  std::vector<size_t> sa_off(P), sb_off(P);
  for(int i = 0; i < P; ++i) {
    const auto& d = g->descs[i];
    if(F::elem != Elem::F16) continue;
    sa_off[i] = off = align_up(off, 256);
    off += size_t((d.M + 63) / 64) * size_t(kp[i] / 64) * 4;
    sb_off[i] = off = align_up(off, 256);
    off += size_t((d.N + 63) / 64) * size_t(kp[i] / 64) * 4;
  }
  const size_t probs_off = align_up(off, 256), maps_off = align_up(probs_off + P * sizeof(GroupProblem), 128);
  std::vector<int4> tiles;
  for(int i = 0; i < P; ++i) {
    const auto& d = g->descs[i];
    const int tm = int((d.M + F::BM - 1) / F::BM), tn = int((d.N + F::BN - 1) / F::BN);
    for(int x = 0; x < tm; ++x)
      for(int y = 0; y < tn; ++y) tiles.push_back(make_int4(i, x, y, 0));
  }
  std::stable_sort(tiles.begin(), tiles.end(), [&](const int4& u, const int4& v) { return kp[u.x] > kp[v.x]; });
  const size_t tiles_off = align_up(maps_off + P * sizeof(ProductMaps), 256);
  const size_t jobs_off = align_up(tiles_off + tiles.size() * sizeof(int4), 256);
  int64_t nblocks = 0;  // split blocks of all operands
  for(int i = 0; i < P; ++i) {
    const auto& d = g->descs[i];
    if(d.M > 0 && d.N > 0) nblocks += ((d.M + 63) / 64 + (d.N + 63) / 64) * (kp[i] / 64);
  }
  if(nblocks >= (1ll << 31)) return fail(GBPOLY_ERR_UNSUPPORTED, "too many split blocks in one grouped plan");
  const size_t table_off = align_up(jobs_off + 2 * P * sizeof(SplitJob), 256);
  const size_t total = table_off + size_t(nblocks) * sizeof(int4);
  GBPOLY_CUDA_TRY(cudaMalloc(&g->dev, total));
  g->dev_bytes = total;
  char* base = static_cast<char*>(g->dev);

  std::vector<GroupProblem> probs(P);
  std::vector<ProductMaps> maps(P);
  std::vector<SplitJob> jobs;
  std::vector<int4> table;  // split block -> (job, row block, k block, 0), operand by operand
  table.reserve(size_t(nblocks));
  auto add_blocks = [&](int64_t rows, int kb) {
    const int job = int(jobs.size()) - 1;
    for(int rb = 0; rb < int((rows + 63) / 64); ++rb)
      for(int k = 0; k < kb; ++k) table.push_back(make_int4(job, rb, k, 0));
  };
  gbpoly_status st;
  for(int i = 0; i < P; ++i) {
    const auto& d = g->descs[i];
    float* const scale_a = F::elem == Elem::F16 ? reinterpret_cast<float*>(base + sa_off[i]) : nullptr;
    float* const scale_b = F::elem == Elem::F16 ? reinterpret_cast<float*>(base + sb_off[i]) : nullptr;
    probs[i] = GroupProblem{int(d.M), int(d.N), int(kp[i]), 0, d.alpha, d.beta, d.C, d.ldc, scale_a, scale_b};
    const size_t sa = align_up(size_t(d.M) * kp[i] * F::esz, 1024), sb = align_up(size_t(d.N) * kp[i] * F::esz, 1024);
    Panels pa{base + a_off[i], sa}, pb{base + b_off[i], sb};
    if(d.M > 0 && d.N > 0) {
      if((st = make_product_maps<F>(ctx, maps[i], pa, d.M, pb, d.N, kp[i])) != GBPOLY_OK) return st;
      const int kb = int(kp[i] / 64);
      jobs.push_back(SplitJob{d.A, d.lda, d.op_a == GBPOLY_OP_N ? 1 : 0, int(d.M), int(d.K), int(kp[i]), pa.base,
          int64_t(sa / F::esz), scale_a});
      add_blocks(d.M, kb);
      jobs.push_back(SplitJob{d.B, d.ldb, d.op_b == GBPOLY_OP_T ? 1 : 0, int(d.N), int(d.K), int(kp[i]), pb.base,
          int64_t(sb / F::esz), scale_b});
      add_blocks(d.N, kb);
    }
    g->flops += 2 * d.M * d.N * d.K;
  }
  g->probs = reinterpret_cast<GroupProblem*>(base + probs_off);
  g->maps = reinterpret_cast<ProductMaps*>(base + maps_off);
  g->tiles = reinterpret_cast<int4*>(base + tiles_off);
  g->jobs = reinterpret_cast<SplitJob*>(base + jobs_off);
  g->split_table = reinterpret_cast<int4*>(base + table_off);
  g->ntiles = int(tiles.size());
  g->njobs = int(jobs.size());
  g->split_blocks = int(table.size());
  if(!table.empty())
    GBPOLY_CUDA_TRY(cudaMemcpy(g->split_table, table.data(), table.size() * sizeof(int4), cudaMemcpyHostToDevice));
  GBPOLY_CUDA_TRY(cudaMemcpy(g->probs, probs.data(), P * sizeof(GroupProblem), cudaMemcpyHostToDevice));
  GBPOLY_CUDA_TRY(cudaMemcpy(g->maps, maps.data(), P * sizeof(ProductMaps), cudaMemcpyHostToDevice));
  if(!tiles.empty())
    GBPOLY_CUDA_TRY(cudaMemcpy(g->tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
  if(!jobs.empty())
    GBPOLY_CUDA_TRY(cudaMemcpy(g->jobs, jobs.data(), jobs.size() * sizeof(SplitJob), cudaMemcpyHostToDevice));
  return GBPOLY_OK;
}

template <class F>
gbpoly_status run_grouped(gbpoly_ctx* ctx, gbpoly_grouped* g, const char* name) {
  using T = typename Term<F::elem>::T;
  if(g->split_blocks > 0) {
    ProfileScope prof(ctx, "grouped_split");
    // persistent: 4 CTAs per SM
    const int ctas = std::min(g->split_blocks, 4 * std::max(1, ctx->sm_count));
    grouped_split_kernel<F::elem, F::terms><<<ctas, 256, 0, ctx->stream>>>(g->jobs, g->split_table, g->split_blocks);
    GBPOLY_CUDA_TRY(cudaGetLastError());
  }
  (void)sizeof(T);
  GroupedSched<F::BM, F::BN> sched{g->probs, g->maps, g->tiles, g->ntiles};
  return launch_tc_kernel<F>(ctx, sched, g->ntiles, name);
}

// Tile configurations of grouped plans: 0 = 1-CTA 128 x 128 tiles (least
// padding of small problems), 1 = CTA pairs on 256 x 256 tiles (a few large
// products, as matmulchain's two independent stages), and for bf16x3 and
// fp16x3 2 = 1-CTA 128 x 256 tiles.  Untuned, a group uses 1 when every problem is
// large enough that 256 x 256 tiles pad it about as little as 128 x 128 ones
// and the group fills at least two rounds of pairs, else 0; the autotuner
// (gbpoly_autotune_grouped) times them per problem class.
using GroupBF16x3_w = FormBF16x3;
using GroupBF16x3 = FormBF16x3_c;
using GroupTF32x3 = FormTF32x3_c;
using GroupBF16x6 = FormBF16x6_b;
using GroupTF32 = FormTF32_c;
using GroupBF16x3_p = FormBF16x3_p;
using GroupTF32x3_p = FormTF32x3_p;
using GroupBF16x6_p = FormBF16x6_p;
using GroupTF32_p = FormTF32_p;
using GroupF16x3 = FormF16x3_c;
using GroupF16x3_p = FormF16x3_p;
using GroupF16x3_w = FormF16x3;

bool grouped_pairs(gbpoly_ctx* ctx, const std::vector<gbpoly_gemm_desc>& descs) {
  double work128 = 0, work256 = 0;
  int64_t pair_tiles = 0;
  for(const auto& d : descs) {
    if(d.M <= 0 || d.N <= 0) continue;
    const double k = double(std::max<int64_t>(d.K, 1));
    work128 += double((d.M + 127) / 128 * 128) * double((d.N + 127) / 128 * 128) * k;
    work256 += double((d.M + 255) / 256 * 256) * double((d.N + 255) / 256 * 256) * k;
    pair_tiles += ((d.M + 255) / 256) * ((d.N + 255) / 256);
  }
  return pair_tiles >= ctx->sm_count && work256 <= 1.05 * work128;
}

}  // namespace

int grouped_config_count(gbpoly_precision prec) {
  switch(prec) {
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_FP16X3: return 3;
  case GBPOLY_PREC_TF32X3:
  case GBPOLY_PREC_BF16X6:
  case GBPOLY_PREC_TF32: return 2;
  default: return 0;
  }
}

int default_grouped_config(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count) {
  if(grouped_config_count(prec) == 0) return 0;
  auto it = ctx->tuned_grouped.find(group_class(prec, descs, count));
  if(it != ctx->tuned_grouped.end() && it->second < grouped_config_count(prec)) return it->second;
  return grouped_pairs(ctx, std::vector<gbpoly_gemm_desc>(descs, descs + count)) ? 1 : 0;
}

}  // namespace gbpoly

extern "C" {

gbpoly_status gbpoly_grouped_plan(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count,
    gbpoly_grouped** out) {
  return gbpoly::grouped_plan_config(ctx, prec, descs, count, -1, out);
}

}  // extern "C"

gbpoly_status gbpoly::grouped_plan_config(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int config, gbpoly_grouped** out) {
  using namespace gbpoly;
  if(!ctx || !out || count < 0 || (count > 0 && !descs)) return fail(GBPOLY_ERR_INVALID, "bad argument");
  *out = nullptr;
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  for(int i = 0; i < count; ++i) {
    const auto& d = descs[i];
    const bool bad_op = (d.op_a != GBPOLY_OP_N && d.op_a != GBPOLY_OP_T) || (d.op_b != GBPOLY_OP_N && d.op_b != GBPOLY_OP_T);
    const int64_t ac = d.op_a == GBPOLY_OP_N ? d.K : d.M, ar = d.op_a == GBPOLY_OP_N ? d.M : d.K;
    const int64_t bc = d.op_b == GBPOLY_OP_N ? d.N : d.K, br = d.op_b == GBPOLY_OP_N ? d.K : d.N;
    if(bad_op || d.M < 0 || d.N < 0 || d.K < 0 || d.M >= (1ll << 31) || d.N >= (1ll << 31) || d.K >= (1ll << 30) ||
        (ar > 0 && ac > 0 && (!d.A || d.lda < ac)) || (br > 0 && bc > 0 && (!d.B || d.ldb < bc)) ||
        (d.M > 0 && d.N > 0 && (!d.C || d.ldc < d.N))) {
      char buf[96];
      snprintf(buf, sizeof buf, "grouped problem %d: bad shape, operation, pointer or leading dimension", i);
      return fail(GBPOLY_ERR_INVALID, buf);
    }
  }
  if(prec != GBPOLY_PREC_FP32 && prec != GBPOLY_PREC_BF16X3 && prec != GBPOLY_PREC_TF32X3 &&
      prec != GBPOLY_PREC_BF16X6 && prec != GBPOLY_PREC_TF32 && prec != GBPOLY_PREC_FP16X3)
    return fail(GBPOLY_ERR_UNSUPPORTED, "precision form not available for grouped calls");
  auto* g = new gbpoly_grouped();
  g->prec = prec;
  g->descs.assign(descs, descs + count);
  if(count == 0) {  // an empty group: no device memory, running it launches nothing
    *out = g;
    return GBPOLY_OK;
  }
  gbpoly_status st = GBPOLY_OK;
  switch(prec) {
  case GBPOLY_PREC_FP32: {
    // per-problem launches; the workspace their K splits need is reserved now
    // so that running the plan (or capturing it) allocates nothing
    size_t ws = 0;
    for(auto& d : g->descs) {
      g->flops += 2 * d.M * d.N * d.K;
      ws = std::max(ws, fp32_split_k_bytes(ctx->sm_count, d.M, d.N, d.K));
    }
    if(ws > 0) st = ensure_workspace(ctx, ws);
    break;
  }
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_TF32X3:
  case GBPOLY_PREC_BF16X6:
  case GBPOLY_PREC_TF32:
  case GBPOLY_PREC_FP16X3:
    g->config = config >= 0 ? config : default_grouped_config(ctx, prec, descs, count);
    if(g->config >= grouped_config_count(prec)) {
      st = fail(GBPOLY_ERR_INVALID, "no such grouped tile configuration");
      break;
    }
    switch(prec * 4 + g->config) {
    case GBPOLY_PREC_BF16X3 * 4: st = plan_grouped<GroupBF16x3>(ctx, g); break;
    case GBPOLY_PREC_BF16X3 * 4 + 1: st = plan_grouped<GroupBF16x3_p>(ctx, g); break;
    case GBPOLY_PREC_BF16X3 * 4 + 2: st = plan_grouped<GroupBF16x3_w>(ctx, g); break;
    case GBPOLY_PREC_TF32X3 * 4: st = plan_grouped<GroupTF32x3>(ctx, g); break;
    case GBPOLY_PREC_TF32X3 * 4 + 1: st = plan_grouped<GroupTF32x3_p>(ctx, g); break;
    case GBPOLY_PREC_BF16X6 * 4: st = plan_grouped<GroupBF16x6>(ctx, g); break;
    case GBPOLY_PREC_BF16X6 * 4 + 1: st = plan_grouped<GroupBF16x6_p>(ctx, g); break;
    case GBPOLY_PREC_TF32 * 4: st = plan_grouped<GroupTF32>(ctx, g); break;
    case GBPOLY_PREC_FP16X3 * 4: st = plan_grouped<GroupF16x3>(ctx, g); break;
    case GBPOLY_PREC_FP16X3 * 4 + 1: st = plan_grouped<GroupF16x3_p>(ctx, g); break;
    case GBPOLY_PREC_FP16X3 * 4 + 2: st = plan_grouped<GroupF16x3_w>(ctx, g); break;
    default: st = plan_grouped<GroupTF32_p>(ctx, g); break;
    }
    break;
  default: st = fail(GBPOLY_ERR_UNSUPPORTED, "precision form not available for grouped calls");
  }
  if(st != GBPOLY_OK) {
    if(g->dev) cudaFree(g->dev);
    delete g;
    return st;
  }
  *out = g;
  return GBPOLY_OK;
}

extern "C" {

gbpoly_status gbpoly_grouped_run(gbpoly_ctx* ctx, gbpoly_grouped* g) {
  using namespace gbpoly;
  if(!ctx || !g) return fail(GBPOLY_ERR_INVALID, "bad argument");
  if(g->descs.empty()) return GBPOLY_OK;
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  switch(g->prec) {
  case GBPOLY_PREC_FP32:
    for(const auto& d : g->descs) {
      GemmF32Args a{};
      a.M = d.M, a.N = d.N, a.K = d.K, a.alpha = d.alpha, a.beta = d.beta, a.op_a = d.op_a, a.op_b = d.op_b;
      a.A = d.A, a.lda = d.lda, a.B = d.B, a.ldb = d.ldb, a.C = d.C, a.ldc = d.ldc;
      gbpoly_status st = launch_gemm_f32_simt(ctx, a);
      if(st != GBPOLY_OK) return st;
    }
    return GBPOLY_OK;
  case GBPOLY_PREC_BF16X3:
    return g->config == 1   ? run_grouped<GroupBF16x3_p>(ctx, g, "grouped_bf16x3_gemm")
           : g->config == 2 ? run_grouped<GroupBF16x3_w>(ctx, g, "grouped_bf16x3_gemm")
                            : run_grouped<GroupBF16x3>(ctx, g, "grouped_bf16x3_gemm");
  case GBPOLY_PREC_TF32X3:
    return g->config == 1 ? run_grouped<GroupTF32x3_p>(ctx, g, "grouped_tf32x3_gemm")
                          : run_grouped<GroupTF32x3>(ctx, g, "grouped_tf32x3_gemm");
  case GBPOLY_PREC_BF16X6:
    return g->config == 1 ? run_grouped<GroupBF16x6_p>(ctx, g, "grouped_bf16x6_gemm")
                          : run_grouped<GroupBF16x6>(ctx, g, "grouped_bf16x6_gemm");
  case GBPOLY_PREC_TF32:
    return g->config == 1 ? run_grouped<GroupTF32_p>(ctx, g, "grouped_tf32_gemm")
                          : run_grouped<GroupTF32>(ctx, g, "grouped_tf32_gemm");
  case GBPOLY_PREC_FP16X3:
    return g->config == 1   ? run_grouped<GroupF16x3_p>(ctx, g, "grouped_fp16x3_gemm")
           : g->config == 2 ? run_grouped<GroupF16x3_w>(ctx, g, "grouped_fp16x3_gemm")
                            : run_grouped<GroupF16x3>(ctx, g, "grouped_fp16x3_gemm");
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision form not available for grouped calls");
  }
}

gbpoly_status gbpoly_grouped_config_of(gbpoly_grouped* g, int* config) {
  if(!g || !config) return gbpoly::fail(GBPOLY_ERR_INVALID, "bad argument");
  *config = g->config;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_grouped_info(gbpoly_grouped* g, int64_t* flops, int* tiles, size_t* device_bytes) {
  if(!g) return gbpoly::fail(GBPOLY_ERR_INVALID, "null plan");
  if(flops) *flops = g->flops;
  if(tiles) *tiles = g->ntiles;
  if(device_bytes) *device_bytes = g->dev_bytes;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_grouped_destroy(gbpoly_ctx* ctx, gbpoly_grouped* g) {
  if(!g) return GBPOLY_OK;
  if(ctx) {
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
  }
  if(g->dev) cudaFree(g->dev);
  delete g;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_gemm_grouped_f32(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count) {
  gbpoly_grouped* g = nullptr;
  gbpoly_status st = gbpoly_grouped_plan(ctx, prec, descs, count, &g);
  if(st != GBPOLY_OK) return st;
  st = gbpoly_grouped_run(ctx, g);
  gbpoly_status st2 = gbpoly_grouped_destroy(ctx, g);  // waits for the launches
  return st != GBPOLY_OK ? st : st2;
}

}  // extern "C"

namespace gbpoly {

// ------------------------------------------------ allocation-free entry point
//
// Some callers may not allocate device memory when they call a contraction:
// code being captured into a CUDA graph in global capture mode (cudaMalloc is
// not permitted there), applications that hand the whole device to their own
// memory pool at start-up, real-time loops that forbid an allocation (it can
// synchronise the device) after initialisation, and processes under a hard
// device-memory quota.  For them the split-BF16 form has a second entry point
// whose split panels live in this fixed, file-scope device array instead of
// the context workspace.  Every GPU that loads this library holds the array
// until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

// Device address of g_noalloc_scratch, looked up with the device current
// (the array's name is only a host-side handle in host code).  The address
// belongs to the device's context: the cache remembers which context it was
// read in and reads it again when the current context differs, as it does
// after cudaDeviceReset has torn the old one down and the module has been
// loaded into a new one.
std::mutex g_noalloc_mutex;
struct NoAllocAddr {
  unsigned long long ctx_id = 0;
  void* ptr = nullptr;
};
NoAllocAddr g_noalloc_addr[64];

gbpoly_status noalloc_scratch(int device, char** out) {
  if(device < 0 || device >= 64) return fail(GBPOLY_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocAddr& slot = g_noalloc_addr[device];
  const unsigned long long id = current_context_id();
  if(!slot.ptr || (id != 0 && id != slot.ctx_id)) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if(e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    slot.ptr = p;
    slot.ctx_id = id;
  }
  *out = static_cast<char*>(slot.ptr);
  return GBPOLY_OK;
}

}  // namespace

gbpoly_status launch_gemm_bf16x3_noalloc(gbpoly_ctx* ctx, const GemmF32Args& a) {
  using F = FormBF16x3;
  if(a.M == 0 || a.N == 0) return GBPOLY_OK;
  if(a.M >= (1ll << 31) || a.N >= (1ll << 31) || a.K >= (1ll << 30))
    return fail(GBPOLY_ERR_UNSUPPORTED, "dimension too large for the tensor-core kernels");
  const bool same = same_operand(a);
  const Layout lay = layout<F>(a.M, a.N, a.K, same);
  const size_t need = lay.a_bytes + lay.b_bytes;
  if(need > kNoAllocScratchBytes) {
    char buf[256];
    snprintf(buf, sizeof buf,
        "M=%lld N=%lld K=%lld needs %zu bytes of split panels; the allocation-free entry point has %zu "
        "(about (M+N) x round_up(K,64) x 4 bytes must fit)",
        (long long)a.M, (long long)a.N, (long long)a.K, need, kNoAllocScratchBytes);
    return fail(GBPOLY_ERR_INVALID, buf);
  }
  char* ws = nullptr;
  gbpoly_status st = noalloc_scratch(ctx->device, &ws);
  if(st != GBPOLY_OK) return st;
  Panels pa{ws, lay.a_stride};
  Panels pb = same ? pa : Panels{ws + lay.a_bytes, lay.b_stride};
  if(a.K > 0) {
    // the split pass writes every panel element it is read from (zero K padding included)
    if((st = launch_split<F>(ctx, a.A, a.lda, a.op_a == GBPOLY_OP_N, a.M, a.K, lay.Kp, pa)) != GBPOLY_OK) return st;
    if(!same && (st = launch_split<F>(ctx, a.B, a.ldb, a.op_b == GBPOLY_OP_T, a.N, a.K, lay.Kp, pb)) != GBPOLY_OK)
      return st;
  } else {
    GBPOLY_CUDA_TRY(cudaMemsetAsync(ws, 0, need, ctx->stream));  // the array keeps the previous call's panels
  }
  GemmMaps maps;
  if((st = make_product_maps<F>(ctx, maps.p[0], pa, a.M, pb, a.N, lay.Kp)) != GBPOLY_OK) return st;
  maps.p[1] = maps.p[0];
  SingleSched<F::BM, F::BN> sched{maps, 1, int(a.M), int(a.N), int(lay.Kp), a.alpha, a.beta, a.C, a.ldc};
  const int64_t tiles = ((a.M + F::BM - 1) / F::BM) * ((a.N + F::BN - 1) / F::BN);
  return launch_tc_kernel<F>(ctx, sched, tiles, "bf16x3_gemm_noalloc");
}

}  // namespace gbpoly

extern "C" gbpoly_status gbpoly_gemm_f32_bf16x3_noalloc(gbpoly_ctx* ctx, gbpoly_op op_a, gbpoly_op op_b, int64_t M,
    int64_t N, int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
    int64_t ldc) {
  using namespace gbpoly;
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
  GemmF32Args a{};
  a.M = M, a.N = N, a.K = K, a.alpha = alpha, a.beta = beta, a.op_a = op_a, a.op_b = op_b;
  a.A = A, a.lda = lda, a.B = B, a.ldb = ldb, a.C = C, a.ldc = ldc;
  return launch_gemm_bf16x3_noalloc(ctx, a);
}
