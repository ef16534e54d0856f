// Internal declarations shared by the gbpoly CUDA translation units.
//
// Device helpers here are hand-written inline PTX for sm_103a: mbarrier
// phases with bounded waits, 2-D TMA tile loads, and the global timer.
// Every wait on an mbarrier gives up after kWaitTimeoutNs, records a code in
// the context's error word (mapped host memory) and lets the kernel return,
// so a broken pipeline never hangs the GPU.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbpoly.h"

namespace gbpoly {

// ------------------------------------------------------------------ host side

// Error word codes written by kernels (first writer wins).
enum DeviceError : int {
  kDevErrNone = 0,
  kDevErrFullWait = 1,    // consumer waited too long for a filled stage
  kDevErrEmptyWait = 2,   // producer waited too long for a drained stage
  kDevErrMmaWait = 3,     // epilogue waited too long for the accumulator
  kDevErrDrainWait = 4,   // teardown waited too long for in-flight copies
  kDevErrTmemAlloc = 5,   // tensor-memory allocation did not fit
  kDevErrSplitWait = 6,   // a K-split tile's first half waited too long for the second
  kDevErrProbeWait = 7,   // gbpoly_wait_probe: a wait on a barrier nothing completes ran out (as intended)
};

struct Workspace {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace gbpoly

namespace gbpoly {
// One launch bracketed by events while profiling is enabled.
struct ProfileRecord {
  const char* kernel;
  cudaEvent_t start, end;
};
}  // namespace gbpoly

struct gbpoly_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int* err_host = nullptr;  // mapped pinned word; kernels write it, host reads after sync
  int* err_dev = nullptr;   // device alias of err_host
  // stream hold (gbpoly_stream_hold/release): mapped pinned word, its device
  // alias and the value the next hold waits for
  unsigned* hold_host = nullptr;
  unsigned* hold_dev = nullptr;
  unsigned hold_value = 0;
  int sm_count = 0;
  int sm_clock_khz = 0;
  int cc_major = 0, cc_minor = 0;
  char name[256] = {0};
  gbpoly::Workspace ws;
  gbpoly::Workspace stats;  // per-chunk column partial sums (colstats.cu)
  gbpoly::Workspace centred;  // gbpoly_covariance_f32, fp32 and fp8 forms: the centred copy of X
  PFN_cuTensorMapEncodeTiled_v12000 encode_tiled = nullptr;
  bool profiling = false;
  bool tail_split = true;  // K-split units for the last round of CTA-pair tiles
  std::vector<gbpoly::ProfileRecord> prof;        // launches since the last read
  std::vector<cudaEvent_t> event_pool;            // reusable events
  // tile configuration per (form, log2-bucket of M, N, K), from the autotuner
  std::map<std::tuple<int, int, int, int>, int> tuned;
  // grouped plans: tile configuration per problem class (form, log2-buckets
  // of the problem count and of the median M, N, K)
  std::map<std::tuple<int, int, int, int, int>, int> tuned_grouped;
  // host-buffer calls: copy streams and device staging of the operands
  cudaStream_t h2d_stream = nullptr, d2h_stream = nullptr;
  void *stage_a = nullptr, *stage_b = nullptr, *stage_c = nullptr;
  size_t stage_a_bytes = 0, stage_b_bytes = 0, stage_c_bytes = 0;
};

namespace gbpoly {

// Thread-local error text, returned by gbpoly_last_error().
void set_error(const std::string& msg);
gbpoly_status fail(gbpoly_status code, const std::string& msg);
gbpoly_status cuda_fail(cudaError_t e, const char* what);

#define GBPOLY_CUDA_TRY(expr)                                  \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if(_e != cudaSuccess) return ::gbpoly::cuda_fail(_e, #expr); \
  } while(0)

// Brackets one kernel launch with events when the context is profiling
// (gbpoly_profile_enable); a no-op otherwise.
class ProfileScope {
public:
  ProfileScope(gbpoly_ctx* ctx, const char* kernel);
  ~ProfileScope();

private:
  gbpoly_ctx* ctx_;
  size_t index_ = size_t(-1);
};

// Process-unique id of the calling thread's current CUDA context
// (cuCtxGetId), 0 when the driver does not report one.
unsigned long long current_context_id();

// Set-up that belongs to a device's context (a kernel's shared-memory
// opt-in, an occupancy figure, a symbol's device address) is done once per
// device and remembered with the id of the context it was done in; after
// cudaDeviceReset the device has a new context, valid() is false again and
// the set-up is repeated.  Devices beyond 31 are never remembered (set-up on
// every call).
class ContextMark {
public:
  bool valid(int device) const {
    return device >= 0 && device < 32 && id_[device].load(std::memory_order_acquire) == current_context_id() + 1;
  }
  void set(int device) {
    if(device >= 0 && device < 32) id_[device].store(current_context_id() + 1, std::memory_order_release);
  }

private:
  std::atomic<unsigned long long> id_[32] = {};  // context id + 1 of the set-up; 0: none
};

// Grow the context workspace to at least `bytes` (synchronises when it grows;
// refused during stream capture).
gbpoly_status ensure_workspace(gbpoly_ctx* ctx, size_t bytes);
// Same rule for another per-context scratch buffer.
gbpoly_status ensure_scratch(gbpoly_ctx* ctx, Workspace& w, size_t bytes, const char* what);

// 2-D tensor map over a row-major matrix of `rows` x `cols` elements with
// leading dimension `ld` (elements), box `box_rows` x `box_cols`.
gbpoly_status make_tmap_2d(gbpoly_ctx* ctx, CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes,
    const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
    CUtensorMapSwizzle swizzle);

// FP32 SIMT entry points (sgemm_simt.cu).
// Per-row transform of op(A) applied by the split pass of the tensor-core
// forms before splitting (covariance, correlation: op(A) = X^T, a row of
// op(A) is a column of X): y = x - mean[r], then, with sd, y = (y / div) / sd[r]
// (the arithmetic of gbpoly_center_columns_f32, so the panels are bitwise
// those of the centred copy).  mean == nullptr: none.
struct RowXform {
  const float* mean = nullptr;
  const float* sd = nullptr;
  float div = 1.f;
};

struct GemmF32Args {
  int64_t M, N, K;
  float alpha, beta;
  gbpoly_op op_a, op_b;
  const float* A;
  int64_t lda;
  const float* B;
  int64_t ldb;
  float* C;
  int64_t ldc;
  // Second product accumulated into the same C (syr2k): A2 (N x K) times B2^T.
  bool dual = false;
  const float* A2 = nullptr;
  int64_t lda2 = 0;
  const float* B2 = nullptr;
  int64_t ldb2 = 0;
  // FP32 only: K split count (0: chosen from the shape; 1: none).  Callers
  // that run a contraction in row panels pass the full shape's split so the
  // panels add K in the same order as the whole call.
  int ksplit = 0;
  // Tensor-core forms, symmetric products only: transform of op(A)'s rows.
  RowXform xf;
};
// op(B) is op(A)^T on the same stored matrix (syrk's A.A^T, covariance's
// X^T.X): the product is symmetric, and one set of split panels serves both
// operands.
inline bool symmetric_operand(const GemmF32Args& a) {
  return !a.dual && a.A == a.B && a.lda == a.ldb && a.M == a.N && a.op_a != a.op_b;
}
gbpoly_status launch_gemm_f32_simt(gbpoly_ctx* ctx, const GemmF32Args& a);
// Workspace of the K split the FP32 kernel uses for grids too small to fill a
// device of `sm_count` SMs (0 when it does not split).
size_t fp32_split_k_bytes(int sm_count, int64_t M, int64_t N, int64_t K);
// The K split count gbpoly_gemm_f32 uses for an FP32 contraction of this
// shape on operands the TMA kernel can read (1: no split).
int fp32_split_k_count(int sm_count, int64_t M, int64_t N, int64_t K);
// Tensor-core forms (split_gemm.cu): tf32, bf16x3, tf32x3, bf16x6, fp16x3,
// fp8.  The split term panels live in the context workspace.
gbpoly_status launch_gemm_tensor(gbpoly_ctx* ctx, gbpoly_precision prec, const GemmF32Args& a);
// Tile configurations of a tensor-core form (0 for none); launch with an
// explicit configuration; the configuration the context uses for a shape.
int tensor_config_count(gbpoly_precision prec);
gbpoly_status launch_gemm_tensor_config(gbpoly_ctx* ctx, gbpoly_precision prec, int config, const GemmF32Args& a);
int tuned_config(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K);
// Configuration used for a shape nobody tuned (split_gemm.cu).
int default_config(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K);
std::tuple<int, int, int, int> shape_bucket(gbpoly_precision prec, int64_t M, int64_t N, int64_t K);
// Row-panel execution of a tensor-core contraction (host-buffer calls): the
// plan fixes form and configuration for the full shape; each panel call
// splits its rows of A (and, for the first panel, all of B) and runs them.
struct TensorPlan {
  gbpoly_precision prec = GBPOLY_PREC_FP32;
  int config = 0;
  int64_t M = 0;
};
gbpoly_status tensor_plan(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op op_a, gbpoly_op op_b, int64_t M, int64_t N,
    int64_t K, TensorPlan* plan);
gbpoly_status tensor_plan_panel(gbpoly_ctx* ctx, const TensorPlan& plan, const GemmF32Args& a, bool first, int64_t r0);
// Grouped plans (split_gemm.cu): the number of tile configurations of a form,
// the problem class a group belongs to (autotune.cu), and planning with a
// given configuration (-1: the tuned one for the class, else the rule).
int grouped_config_count(gbpoly_precision prec);
std::tuple<int, int, int, int, int> group_class(gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count);
int default_grouped_config(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count);
gbpoly_status grouped_plan_config(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count,
    int config, gbpoly_grouped** out);
// Workspace bytes launch_gemm_tensor needs for this shape (0 for FP32).
size_t workspace_bytes(gbpoly_precision prec, int64_t M, int64_t N, int64_t K, bool same_operand);

// ---------------------------------------------------------------- device side

constexpr unsigned long long kWaitTimeoutNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_timer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of `bar` to complete.  Returns false (after
// recording `code` in *err) if it does not within `limit_ns`, or as soon as
// another thread of the grid has recorded an error.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, int* err, int code,
    unsigned long long limit_ns) {
  if(mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_timer_ns();
  while(true) {
#pragma unroll 1
    for(int i = 0; i < 32; ++i)
      if(mbar_try_wait(bar, parity)) return true;
    if(*reinterpret_cast<volatile int*>(err) != 0) return false;
    if(global_timer_ns() - t0 > limit_ns) {
      atomicCAS(err, 0, code);
      return false;
    }
  }
}

// The kernels' waits: mbar_wait_for with the library-wide limit kWaitTimeoutNs.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  return mbar_wait_for(bar, parity, err, code, kWaitTimeoutNs);
}

// Wait until the global counter reaches `target` (other CTAs of the same
// launch add to it).  Bounded like mbar_wait; ordered before the caller's
// later loads on success.
__device__ __forceinline__ bool wait_count(const int* counter, int target, int* err, int code) {
  const volatile int* c = counter;
  const uint64_t t0 = global_timer_ns();
  for(int n = 0; *c < target; ++n) {
    __nanosleep(128);
    if((n & 15) == 15) {
      if(*reinterpret_cast<volatile int*>(err) != 0) return false;
      if(global_timer_ns() - t0 > kWaitTimeoutNs) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
  __threadfence();
  return true;
}

// Fetch the 128-byte line holding p into L2 (no register or shared-memory cost).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------- thread-block clusters
// Rank of this CTA in its cluster, the cluster's index and the number of
// clusters of the grid (x dimension).
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count_x() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// Every thread of every CTA of the cluster (release / acquire).
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_map(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
// Arrive on an mbarrier given by its cluster address (this CTA's or a
// peer's), with the default (CTA-scope) release: the arrival only counts,
// the data it stands for (tensor-memory reads) is ordered by tcgen05 fences.
// A cluster-scope release would make the arriving warp wait for all its
// outstanding global stores first.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster_addr) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster_addr) : "memory");
}

// TMA load of a CTA pair: the box lands in this CTA's `dst`, the transaction
// bytes are signalled on an mbarrier of either CTA of the pair (its cluster
// address).
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cluster_addr, int x,
    int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster_addr), "r"(x), "r"(y)
      : "memory");
}

// 2-D tiled TMA load: box at (x = innermost coordinate, y) into smem `dst`,
// completion signalled as transaction bytes on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

// TMA store of a 2-D box from shared memory (bulk-group completion), and the
// waits on this thread's bulk groups: until their shared-memory reads are
// done (the buffer may be rewritten), or until they are complete.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
      "r"(smem_u32(src)), "r"(x), "r"(y)
      : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace gbpoly
