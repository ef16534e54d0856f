// Hand-written PTX wrappers for the sm_100-family tensor-core path (tcgen05):
// tensor-memory allocation, MMA issue and commit, TMEM -> register loads,
// and the shared-memory / instruction descriptors the MMA consumes.
//
// Descriptor formats (PTX ISA, "tcgen05 shared memory descriptor" and
// "instruction descriptor"):
//   shared memory descriptor, 64 bit:
//     [0,14)  start address >> 4        [16,30) leading byte offset >> 4
//     [32,46) stride byte offset >> 4   [46,48) version (1 on sm_100 family)
//     [49,52) base offset               [52]    LBO mode
//     [61,64) layout: 0 none, 2 SWIZZLE_128B, 4 SWIZZLE_64B, 6 SWIZZLE_32B
//   instruction descriptor for kind::f16 / kind::tf32, 32 bit:
//     [4,6) D format (1 = F32)   [7,10) A format   [10,13) B format
//           (kind::f16: 0 F16, 1 BF16; kind::tf32: 2 TF32)
//     [13] negate A  [14] negate B  [15] A MN-major  [16] B MN-major
//     [17,23) N >> 3             [24,29) M >> 4
#pragma once

#include <stdint.h>

namespace gbpoly {
namespace umma {

// K-major operand tile written by TMA with 128-byte swizzle: rows of 128
// bytes, 8-row swizzle atoms of 1024 bytes (stride byte offset), tile base
// 1024-byte aligned.  The leading byte offset is unused for swizzled K-major
// layouts.  Advancing along K inside the atom is done by adding the byte
// offset to the start address.
__device__ __forceinline__ uint64_t desc_k_sw128(uint32_t smem_addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((smem_addr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;           // LBO (unused), encoded 16 bytes
  d |= static_cast<uint64_t>(1024 >> 4) << 32;   // SBO: 8 rows x 128 B
  d |= static_cast<uint64_t>(1) << 46;           // version
  d |= static_cast<uint64_t>(2) << 61;           // SWIZZLE_128B
  return d;
}

// Same for 64-byte rows written with 64-byte swizzle (8-row atoms of 512 bytes).
__device__ __forceinline__ uint64_t desc_k_sw64(uint32_t smem_addr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((smem_addr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;           // LBO (unused)
  d |= static_cast<uint64_t>(512 >> 4) << 32;    // SBO: 8 rows x 64 B
  d |= static_cast<uint64_t>(1) << 46;           // version
  d |= static_cast<uint64_t>(4) << 61;           // SWIZZLE_64B
  return d;
}

// K-major swizzled operand descriptor for ROW-byte rows (128 or 64).
template <int ROW>
__device__ __forceinline__ uint64_t desc_k(uint32_t smem_addr) {
  static_assert(ROW == 128 || ROW == 64, "row bytes");
  if constexpr(ROW == 128)
    return desc_k_sw128(smem_addr);
  else
    return desc_k_sw64(smem_addr);
}

enum class AbType : uint32_t { F16 = 0, BF16 = 1, TF32 = 2 };

template <int M, int N, AbType T>
struct InstrDesc {
  static_assert(M == 64 || M == 128 || M == 256, "UMMA M");
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "UMMA N");
  static constexpr uint32_t value = (1u << 4) | (static_cast<uint32_t>(T) << 7) | (static_cast<uint32_t>(T) << 10) |
                                    (static_cast<uint32_t>(N >> 3) << 17) | (static_cast<uint32_t>(M >> 4) << 24);
};

// Instruction descriptor for kind::f8f6f4 with E4M3 operands (format code 0)
// and FP32 accumulation: same field positions as kind::f16.
template <int M, int N>
struct InstrDescE4M3 {
  static_assert(M == 64 || M == 128, "UMMA M");
  static_assert(N % 16 == 0 && N >= 16 && N <= 256, "UMMA N");
  static constexpr uint32_t value = (1u << 4) | (static_cast<uint32_t>(N >> 3) << 17) |
                                    (static_cast<uint32_t>(M >> 4) << 24);
};

// ---------------------------------------------------------------- TMEM alloc
// Executed by all 32 lanes of one warp.  Writes the base address to smem.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ------------------------------------------------------------------- MMA ---
// D[tmem] (+)= A[smem desc] * B[smem desc]^T, kind::f16, one CTA.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A * B^T, kind::tf32 (FP32 operands in shared memory).
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// D[tmem] (+)= A * B^T, kind::f8f6f4 (8-bit operands, K = 32 per instruction).
__device__ __forceinline__ void mma_f8(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// ------------------------------------------------------------ CTA pairs --
// cta_group::2: one warp in EACH CTA of the pair executes the allocation
// instructions; the pair gets the same TMEM columns in both CTAs.
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish_pair() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// D (M = 256 over the pair: 128 rows in each CTA's TMEM) (+)= A * B^T, issued by
// one thread of the pair's first CTA; A and B descriptors name the same
// shared-memory offsets in both CTAs (each CTA holds half of A's rows and
// half of B's rows).
__device__ __forceinline__ void mma_f16_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_tf32_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
    uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// Arrive on the mbarrier at `bar`'s offset in every CTA of `cta_mask` once
// the pair MMAs issued so far by this thread have completed.
__device__ __forceinline__ void commit_pair(uint64_t* bar, uint16_t cta_mask) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"(cta_mask)
      : "memory");
}

// Arrive on `bar` once every tcgen05 operation issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// ------------------------------------------------------------- TMEM loads --
// 32 lanes x 32 columns of 32-bit: thread t of the warp receives lane
// (taddr.lane + t), columns [taddr.col, taddr.col + 32).
__device__ __forceinline__ void tmem_ld_32x32b_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

// Per-warpgroup register budget (all 128 threads of the warpgroup execute it).
template <uint32_t N>
__device__ __forceinline__ void regs_increase() {
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(N));
}
template <uint32_t N>
__device__ __forceinline__ void regs_decrease() {
  asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(N));
}

__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace umma
}  // namespace gbpoly
