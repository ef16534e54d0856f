// C ABI of libgbpoly: context, memory, events and the contraction entry
// points declared in include/gbpoly.h.  Argument checking lives here; the
// kernels live in their own translation units.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <string>

#include "gbpoly_internal.cuh"

namespace gbpoly {

namespace {
thread_local std::string g_last_error;
}

const char* last_error_cstr() { return g_last_error.c_str(); }

void set_error(const std::string& msg) { g_last_error = msg; }

gbpoly_status fail(gbpoly_status code, const std::string& msg) {
  set_error(msg);
  return code;
}

gbpoly_status cuda_fail(cudaError_t e, const char* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  set_error(msg);
  return (e == cudaErrorMemoryAllocation) ? GBPOLY_ERR_NOMEM : GBPOLY_ERR_CUDA;
}

gbpoly_status ensure_scratch(gbpoly_ctx* ctx, Workspace& w, size_t bytes, const char* what) {
  if(w.bytes >= bytes) return GBPOLY_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GBPOLY_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cs));
  if(cs != cudaStreamCaptureStatusNone)
    return fail(GBPOLY_ERR_STATE, std::string(what) + " would grow during graph capture; make the same call once "
                                                      "before capturing (or call gbpoly_workspace_reserve)");
  if(w.ptr) {
    GBPOLY_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    GBPOLY_CUDA_TRY(cudaFree(w.ptr));
    w.ptr = nullptr;
    w.bytes = 0;
  }
  const size_t rounded = (bytes + (size_t(1) << 21) - 1) & ~((size_t(1) << 21) - 1);
  GBPOLY_CUDA_TRY(cudaMalloc(&w.ptr, rounded));
  w.bytes = rounded;
  return GBPOLY_OK;
}

gbpoly_status ensure_workspace(gbpoly_ctx* ctx, size_t bytes) { return ensure_scratch(ctx, ctx->ws, bytes, "workspace"); }

namespace {
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);
std::atomic<PfnCtxGetCurrent> g_ctx_get_current{nullptr};
std::atomic<PfnCtxGetId> g_ctx_get_id{nullptr};
std::atomic<bool> g_ctx_fns_resolved{false};
}  // namespace

unsigned long long current_context_id() {
  if(!g_ctx_fns_resolved.load(std::memory_order_acquire)) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_current.store(reinterpret_cast<PfnCtxGetCurrent>(fn));
    fn = nullptr;
    if(cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_get_id.store(reinterpret_cast<PfnCtxGetId>(fn));
    g_ctx_fns_resolved.store(true, std::memory_order_release);
  }
  const PfnCtxGetCurrent get_current = g_ctx_get_current.load();
  const PfnCtxGetId get_id = g_ctx_get_id.load();
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if(!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

namespace {
cudaEvent_t pooled_event(gbpoly_ctx* ctx) {
  if(!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if(cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}
}  // namespace

ProfileScope::ProfileScope(gbpoly_ctx* ctx, const char* kernel) : ctx_(ctx) {
  if(!ctx->profiling) return;
  ProfileRecord r{kernel, pooled_event(ctx), pooled_event(ctx)};
  if(!r.start || !r.end) return;
  cudaEventRecord(r.start, ctx->stream);
  index_ = ctx->prof.size();
  ctx->prof.push_back(r);
}

ProfileScope::~ProfileScope() {
  if(index_ != size_t(-1)) cudaEventRecord(ctx_->prof[index_].end, ctx_->stream);
}

gbpoly_status make_tmap_2d(gbpoly_ctx* ctx, CUtensorMap* map, CUtensorMapDataType dtype, size_t elem_bytes,
    const void* base, uint64_t rows, uint64_t cols, uint64_t ld, uint32_t box_rows, uint32_t box_cols,
    CUtensorMapSwizzle swizzle) {
  if(!ctx->encode_tiled) return fail(GBPOLY_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {ld * elem_bytes};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = ctx->encode_tiled(map, dtype, 2, const_cast<void*>(base), dims, strides, box, estr,
      CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if(r != CUDA_SUCCESS) {
    char buf[256];
    snprintf(buf, sizeof buf,
        "cuTensorMapEncodeTiled failed (%d): rows=%llu cols=%llu ld=%llu box=%ux%u elem=%zu base=%p", int(r),
        (unsigned long long)rows, (unsigned long long)cols, (unsigned long long)ld, box_rows, box_cols, elem_bytes,
        base);
    return fail(GBPOLY_ERR_INVALID, buf);
  }
  return GBPOLY_OK;
}

// Holds the stream until the host stores `value` into the mapped word, or
// until `timeout_ns` have passed (a hold nobody releases ends by itself).
__global__ void hold_kernel(const volatile unsigned* word, unsigned value, uint64_t timeout_ns) {
  if(threadIdx.x != 0) return;
  const uint64_t t0 = global_timer_ns();
  while(int(*word - value) < 0) {
    if(global_timer_ns() - t0 > timeout_ns) return;
    __nanosleep(256);
  }
}

// gbpoly_wait_probe: one bounded wait, through the kernels' own wait
// routine, on an mbarrier whose phase nothing completes.  It runs out after
// limit_ns, records kDevErrProbeWait in the error word and returns, as a
// kernel whose pipeline stalled does; no copy or MMA is in flight.
__global__ void wait_probe_kernel(int* err, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if(threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if(threadIdx.x == 0) mbar_wait_for(&bar, 0, err, kDevErrProbeWait, limit_ns);
  __syncthreads();
}

// ------------------------------------------------------ host fault injection
// GBPOLY_FAULT_INJECT, read when a context is created, makes one host-side
// call fail or misbehave so that callers can test their error paths without
// any fault on the GPU:
//   alloc:N    the N-th later gbpoly_malloc (process-wide) returns
//              GBPOLY_ERR_NOMEM without calling cudaMalloc;
//   corrupt:N  after the N-th later gbpoly_memcpy_d2h has landed, a host
//              callback on the stream changes the first 4 bytes of its
//              destination (read as a float v, written as 2v + 1).
// Unset (or any other value) clears a pending injection.
namespace {
std::atomic<long> g_inject_alloc{0}, g_inject_corrupt{0};

void read_fault_injection() {
  g_inject_alloc = 0;
  g_inject_corrupt = 0;
  const char* v = getenv("GBPOLY_FAULT_INJECT");
  if(!v) return;
  long n = 0;
  if(sscanf(v, "alloc:%ld", &n) == 1 && n > 0) g_inject_alloc = n;
  else if(sscanf(v, "corrupt:%ld", &n) == 1 && n > 0) g_inject_corrupt = n;
}

// true exactly once: when the countdown steps from 1 to 0
bool inject_now(std::atomic<long>& countdown) {
  long c = countdown.load();
  while(c > 0)
    if(countdown.compare_exchange_weak(c, c - 1)) return c == 1;
  return false;
}

void CUDART_CB corrupt_first_float(void* p) {
  float v;
  memcpy(&v, p, sizeof v);
  v = 2.0f * v + 1.0f;
  memcpy(p, &v, sizeof v);
}
}  // namespace

}  // namespace gbpoly

using namespace gbpoly;

namespace {

gbpoly_status check_ctx(gbpoly_ctx* ctx) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if(e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return GBPOLY_OK;
}

#define CTX_TRY(ctx)                               \
  do {                                             \
    gbpoly_status _s = check_ctx(ctx);             \
    if(_s != GBPOLY_OK) return _s;                 \
  } while(0)

gbpoly_status check_matrix(const char* name, const void* p, int64_t rows, int64_t cols, int64_t ld) {
  if(rows < 0 || cols < 0) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": negative dimension");
  if(rows > 0 && cols > 0) {
    if(!p) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": null pointer");
    if(ld < cols) return fail(GBPOLY_ERR_INVALID, std::string(name) + ": leading dimension smaller than columns");
  }
  return GBPOLY_OK;
}

}  // namespace

struct gbpoly_event {
  cudaEvent_t ev = nullptr;
};

struct gbpoly_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

const char* gbpoly_last_error(void) { return last_error_cstr(); }

gbpoly_status gbpoly_init(int device, gbpoly_ctx** out_ctx) {
  if(!out_ctx) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *out_ctx = nullptr;
  read_fault_injection();
  int count = 0;
  GBPOLY_CUDA_TRY(cudaGetDeviceCount(&count));
  if(device < 0 || device >= count) return fail(GBPOLY_ERR_INVALID, "device index out of range");
  GBPOLY_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  GBPOLY_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  auto* ctx = new gbpoly_ctx();
  ctx->device = device;
  ctx->sm_count = prop.multiProcessorCount;
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
  ctx->sm_clock_khz = clk;
  ctx->cc_major = prop.major;
  ctx->cc_minor = prop.minor;
  strncpy(ctx->name, prop.name, sizeof(ctx->name) - 1);
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if(e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->err_host), sizeof(int), cudaHostAllocMapped);
  if(e == cudaSuccess) {
    *ctx->err_host = 0;
    e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->err_dev), ctx->err_host, 0);
  }
  if(e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->hold_host), sizeof(unsigned), cudaHostAllocMapped);
  if(e == cudaSuccess) {
    *ctx->hold_host = 0;
    e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->hold_dev), ctx->hold_host, 0);
  }
  if(e != cudaSuccess) {
    gbpoly_status st = cuda_fail(e, "context setup");
    if(ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if(ctx->err_host) cudaFreeHost(ctx->err_host);
    if(ctx->hold_host) cudaFreeHost(ctx->hold_host);
    delete ctx;
    return st;
  }
  ctx->stream = ctx->own_stream;
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    ctx->encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  *out_ctx = ctx;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_destroy(gbpoly_ctx* ctx) {
  if(!ctx) return GBPOLY_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if(ctx->ws.ptr) cudaFree(ctx->ws.ptr);
  if(ctx->stats.ptr) cudaFree(ctx->stats.ptr);
  if(ctx->centred.ptr) cudaFree(ctx->centred.ptr);
  for(void* p : {ctx->stage_a, ctx->stage_b, ctx->stage_c})
    if(p) cudaFree(p);
  if(ctx->h2d_stream) cudaStreamDestroy(ctx->h2d_stream);
  if(ctx->d2h_stream) cudaStreamDestroy(ctx->d2h_stream);
  for(auto& r : ctx->prof) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.end);
  }
  for(auto e : ctx->event_pool) cudaEventDestroy(e);
  if(ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  if(ctx->err_host) cudaFreeHost(ctx->err_host);
  if(ctx->hold_host) cudaFreeHost(ctx->hold_host);
  delete ctx;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_device_name(gbpoly_ctx* ctx, char* buf, size_t buflen) {
  if(!ctx || !buf || buflen == 0) return fail(GBPOLY_ERR_INVALID, "bad argument");
  strncpy(buf, ctx->name, buflen - 1);
  buf[buflen - 1] = 0;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_device_props(gbpoly_ctx* ctx, int* sm_count, int* sm_clock_khz, int* cc_major, int* cc_minor) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  if(sm_count) *sm_count = ctx->sm_count;
  if(sm_clock_khz) *sm_clock_khz = ctx->sm_clock_khz;
  if(cc_major) *cc_major = ctx->cc_major;
  if(cc_minor) *cc_minor = ctx->cc_minor;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_synchronize(gbpoly_ctx* ctx) {
  CTX_TRY(ctx);
  GBPOLY_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  const int code = *reinterpret_cast<volatile int*>(ctx->err_host);
  if(code != 0) {
    *reinterpret_cast<volatile int*>(ctx->err_host) = 0;
    char buf[160];
    snprintf(buf, sizeof buf, "a device-side bounded wait timed out (code %d); the kernel returned early", code);
    return fail(GBPOLY_ERR_TIMEOUT, buf);
  }
  return GBPOLY_OK;
}

gbpoly_status gbpoly_set_stream(gbpoly_ctx* ctx, void* cuda_stream) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  ctx->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->own_stream;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_profile_enable(gbpoly_ctx* ctx, int enable) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  ctx->profiling = enable != 0;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_tail_split_enable(gbpoly_ctx* ctx, int enable) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  ctx->tail_split = enable != 0;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_profile_read(gbpoly_ctx* ctx, int max_entries, char* names, int* counts, double* total_ms,
    int* n_entries) {
  CTX_TRY(ctx);
  if(max_entries < 0 || (max_entries > 0 && (!names || !counts || !total_ms)) || !n_entries)
    return fail(GBPOLY_ERR_INVALID, "bad argument");
  GBPOLY_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  std::vector<std::string> keys;
  std::vector<int> cnt;
  std::vector<double> tot;
  for(auto& r : ctx->prof) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.start, r.end);
    size_t i = 0;
    while(i < keys.size() && keys[i] != r.kernel) ++i;
    if(i == keys.size()) {
      keys.push_back(r.kernel);
      cnt.push_back(0);
      tot.push_back(0.0);
    }
    cnt[i] += 1;
    tot[i] += ms;
    ctx->event_pool.push_back(r.start);
    ctx->event_pool.push_back(r.end);
  }
  ctx->prof.clear();
  *n_entries = int(keys.size());
  for(int i = 0; i < int(keys.size()) && i < max_entries; ++i) {
    strncpy(names + 64 * i, keys[i].c_str(), 63);
    names[64 * i + 63] = 0;
    counts[i] = cnt[i];
    total_ms[i] = tot[i];
  }
  return GBPOLY_OK;
}

gbpoly_status gbpoly_workspace_reserve(gbpoly_ctx* ctx, size_t bytes) {
  CTX_TRY(ctx);
  return ensure_workspace(ctx, bytes);
}

gbpoly_status gbpoly_workspace_query(gbpoly_precision prec, int64_t M, int64_t N, int64_t K, int same_operand,
    size_t* bytes) {
  if(!bytes || M < 0 || N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "bad argument");
  *bytes = workspace_bytes(prec, M, N, K, same_operand != 0);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_graph_begin(gbpoly_ctx* ctx) {
  CTX_TRY(ctx);
  GBPOLY_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_graph_end(gbpoly_ctx* ctx, gbpoly_graph** out) {
  CTX_TRY(ctx);
  if(!out) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *out = nullptr;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GBPOLY_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cs));
  if(cs != cudaStreamCaptureStatusActive) return fail(GBPOLY_ERR_STATE, "no graph capture in progress");
  auto* g = new gbpoly_graph();
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g->graph);
  if(e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if(e != cudaSuccess) {
    if(g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(e, "graph capture");
  }
  *out = g;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_graph_launch(gbpoly_ctx* ctx, gbpoly_graph* g) {
  CTX_TRY(ctx);
  if(!g || !g->exec) return fail(GBPOLY_ERR_INVALID, "null graph");
  ProfileScope prof(ctx, "graph");
  GBPOLY_CUDA_TRY(cudaGraphLaunch(g->exec, ctx->stream));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_graph_destroy(gbpoly_ctx* ctx, gbpoly_graph* g) {
  if(!g) return GBPOLY_OK;
  if(ctx) cudaSetDevice(ctx->device);
  if(g->exec) cudaGraphExecDestroy(g->exec);
  if(g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_malloc(gbpoly_ctx* ctx, void** dptr, size_t bytes) {
  CTX_TRY(ctx);
  if(!dptr) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *dptr = nullptr;
  if(bytes == 0) return GBPOLY_OK;
  if(inject_now(g_inject_alloc))
    return fail(GBPOLY_ERR_NOMEM, "cudaMalloc(dptr, bytes): allocation failure injected by GBPOLY_FAULT_INJECT");
  GBPOLY_CUDA_TRY(cudaMalloc(dptr, bytes));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_free(gbpoly_ctx* ctx, void* dptr) {
  CTX_TRY(ctx);
  if(dptr) GBPOLY_CUDA_TRY(cudaFree(dptr));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_host_alloc(gbpoly_ctx* ctx, void** hptr, size_t bytes) {
  CTX_TRY(ctx);
  if(!hptr) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *hptr = nullptr;
  if(bytes == 0) return GBPOLY_OK;
  GBPOLY_CUDA_TRY(cudaHostAlloc(hptr, bytes, cudaHostAllocDefault));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_host_free(gbpoly_ctx* ctx, void* hptr) {
  CTX_TRY(ctx);
  if(hptr) GBPOLY_CUDA_TRY(cudaFreeHost(hptr));
  return GBPOLY_OK;
}

static gbpoly_status copy(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
  CTX_TRY(ctx);
  if(bytes == 0) return GBPOLY_OK;
  if(!dst || !src) return fail(GBPOLY_ERR_INVALID, "null copy pointer");
  GBPOLY_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, kind, ctx->stream));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_memcpy_h2d(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes) {
  return copy(ctx, dst, src, bytes, cudaMemcpyHostToDevice);
}
gbpoly_status gbpoly_memcpy_d2h(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes) {
  gbpoly_status st = copy(ctx, dst, src, bytes, cudaMemcpyDeviceToHost);
  if(st == GBPOLY_OK && bytes >= sizeof(float) && inject_now(g_inject_corrupt))
    GBPOLY_CUDA_TRY(cudaLaunchHostFunc(ctx->stream, corrupt_first_float, dst));
  return st;
}
gbpoly_status gbpoly_memcpy_d2d(gbpoly_ctx* ctx, void* dst, const void* src, size_t bytes) {
  return copy(ctx, dst, src, bytes, cudaMemcpyDeviceToDevice);
}

gbpoly_status gbpoly_memset(gbpoly_ctx* ctx, void* dst, int value, size_t bytes) {
  CTX_TRY(ctx);
  if(bytes == 0) return GBPOLY_OK;
  if(!dst) return fail(GBPOLY_ERR_INVALID, "null pointer");
  GBPOLY_CUDA_TRY(cudaMemsetAsync(dst, value, bytes, ctx->stream));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_event_create(gbpoly_ctx* ctx, gbpoly_event** ev) {
  CTX_TRY(ctx);
  if(!ev) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  auto* e = new gbpoly_event();
  cudaError_t r = cudaEventCreate(&e->ev);
  if(r != cudaSuccess) {
    delete e;
    return cuda_fail(r, "cudaEventCreate");
  }
  *ev = e;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_event_destroy(gbpoly_ctx* ctx, gbpoly_event* ev) {
  CTX_TRY(ctx);
  if(ev) {
    cudaEventDestroy(ev->ev);
    delete ev;
  }
  return GBPOLY_OK;
}

gbpoly_status gbpoly_event_record(gbpoly_ctx* ctx, gbpoly_event* ev) {
  CTX_TRY(ctx);
  if(!ev) return fail(GBPOLY_ERR_INVALID, "null event");
  GBPOLY_CUDA_TRY(cudaEventRecord(ev->ev, ctx->stream));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_event_elapsed_ms(gbpoly_ctx* ctx, gbpoly_event* start, gbpoly_event* end, float* ms) {
  CTX_TRY(ctx);
  if(!start || !end || !ms) return fail(GBPOLY_ERR_INVALID, "null argument");
  GBPOLY_CUDA_TRY(cudaEventSynchronize(end->ev));
  GBPOLY_CUDA_TRY(cudaEventElapsedTime(ms, start->ev, end->ev));
  return GBPOLY_OK;
}

gbpoly_status gbpoly_stream_hold(gbpoly_ctx* ctx, uint32_t timeout_us) {
  CTX_TRY(ctx);
  const unsigned value = ++ctx->hold_value;
  hold_kernel<<<1, 32, 0, ctx->stream>>>(ctx->hold_dev, value, uint64_t(timeout_us) * 1000ull);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

gbpoly_status gbpoly_wait_probe(gbpoly_ctx* ctx, uint32_t limit_us) {
  CTX_TRY(ctx);
  wait_probe_kernel<<<1, 32, 0, ctx->stream>>>(ctx->err_dev, uint64_t(limit_us) * 1000ull);
  GBPOLY_CUDA_TRY(cudaGetLastError());
  return GBPOLY_OK;
}

gbpoly_status gbpoly_stream_release(gbpoly_ctx* ctx) {
  CTX_TRY(ctx);
  __atomic_store_n(ctx->hold_host, ctx->hold_value, __ATOMIC_RELEASE);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_gemm_f32(gbpoly_ctx* ctx, gbpoly_precision prec, gbpoly_op op_a, gbpoly_op op_b, int64_t M,
    int64_t N, int64_t K, float alpha, const float* A, int64_t lda, const float* B, int64_t ldb, float beta,
    float* C, int64_t ldc) {
  CTX_TRY(ctx);
  if((op_a != GBPOLY_OP_N && op_a != GBPOLY_OP_T) || (op_b != GBPOLY_OP_N && op_b != GBPOLY_OP_T))
    return fail(GBPOLY_ERR_INVALID, "bad operand op");
  if(M < 0 || N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  gbpoly_status st;
  if((st = check_matrix("A", A, op_a == GBPOLY_OP_N ? M : K, op_a == GBPOLY_OP_N ? K : M, lda)) != GBPOLY_OK) return st;
  if((st = check_matrix("B", B, op_b == GBPOLY_OP_N ? K : N, op_b == GBPOLY_OP_N ? N : K, ldb)) != GBPOLY_OK) return st;
  if((st = check_matrix("C", C, M, N, ldc)) != GBPOLY_OK) return st;
  GemmF32Args a{};
  a.M = M, a.N = N, a.K = K, a.alpha = alpha, a.beta = beta, a.op_a = op_a, a.op_b = op_b;
  a.A = A, a.lda = lda, a.B = B, a.ldb = ldb, a.C = C, a.ldc = ldc;
  switch(prec) {
  case GBPOLY_PREC_FP32: return launch_gemm_f32_simt(ctx, a);
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_TF32:
  case GBPOLY_PREC_TF32X3:
  case GBPOLY_PREC_BF16X6:
  case GBPOLY_PREC_FP16X3:
  case GBPOLY_PREC_FP8: return launch_gemm_tensor(ctx, prec, a);
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision not available in this build");
  }
}

gbpoly_status gbpoly_syrk_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t N, int64_t K, float alpha,
    const float* A, int64_t lda, float beta, float* C, int64_t ldc) {
  return gbpoly_gemm_f32(ctx, prec, GBPOLY_OP_N, GBPOLY_OP_T, N, N, K, alpha, A, lda, A, lda, beta, C, ldc);
}

gbpoly_status gbpoly_syr2k_f32(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t N, int64_t K, float alpha,
    const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc) {
  CTX_TRY(ctx);
  gbpoly_status st;
  if(N < 0 || K < 0) return fail(GBPOLY_ERR_INVALID, "negative dimension");
  if((st = check_matrix("A", A, N, K, lda)) != GBPOLY_OK) return st;
  if((st = check_matrix("B", B, N, K, ldb)) != GBPOLY_OK) return st;
  if((st = check_matrix("C", C, N, N, ldc)) != GBPOLY_OK) return st;
  GemmF32Args a{};
  a.M = N, a.N = N, a.K = K, a.alpha = alpha, a.beta = beta, a.op_a = GBPOLY_OP_N, a.op_b = GBPOLY_OP_T;
  a.A = A, a.lda = lda, a.B = B, a.ldb = ldb, a.C = C, a.ldc = ldc;
  a.dual = true, a.A2 = B, a.lda2 = ldb, a.B2 = A, a.ldb2 = lda;
  switch(prec) {
  case GBPOLY_PREC_FP32: return launch_gemm_f32_simt(ctx, a);
  case GBPOLY_PREC_BF16X3:
  case GBPOLY_PREC_TF32:
  case GBPOLY_PREC_TF32X3:
  case GBPOLY_PREC_BF16X6:
  case GBPOLY_PREC_FP16X3:
  case GBPOLY_PREC_FP8: return launch_gemm_tensor(ctx, prec, a);
  default: return fail(GBPOLY_ERR_UNSUPPORTED, "precision not available in this build");
  }
}

}  // extern "C"
