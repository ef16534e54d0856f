// Tile-configuration autotuner for the tensor-core forms.
//
// Each form has a few compiled tile configurations (BN, K bytes per stage and
// swizzle width, pipeline depth; see split_gemm.cu).  The context keeps the
// chosen configuration per (form, ceil(log2) of M, N and K); the autotuner
// times every configuration on the device for a shape and records the
// fastest.  The table can be written to and read from a text file, keyed by
// device name and driver version, so a tuned machine does not tune again.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>

#include "gbpoly_internal.cuh"

namespace gbpoly {

namespace {
int ceil_log2(int64_t x) {
  int l = 0;
  while((int64_t(1) << l) < x && l < 62) ++l;
  return l;
}

__global__ void fill_kernel(float* p, int64_t n, uint32_t seed) {
  for(int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    uint32_t h = uint32_t(i) * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    p[i] = float(h & 0xFFFFFF) * (1.0f / 16777216.0f) - 0.5f;
  }
}

std::string device_key(gbpoly_ctx* ctx) {
  int drv = 0;
  cudaDriverGetVersion(&drv);
  std::string name(ctx->name);
  for(char& c : name)
    if(c == '\t' || c == '\n') c = ' ';
  return name + " driver " + std::to_string(drv);
}
}  // namespace

std::tuple<int, int, int, int> shape_bucket(gbpoly_precision prec, int64_t M, int64_t N, int64_t K) {
  return std::make_tuple(int(prec), ceil_log2(M), ceil_log2(N), ceil_log2(K));
}

int tuned_config(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K) {
  auto it = ctx->tuned.find(shape_bucket(prec, M, N, K));
  return it == ctx->tuned.end() ? default_config(ctx, prec, M, N, K) : it->second;
}

// Problem class of a group: ceil(log2) of the problem count and of the
// median M, N and K (problems with an empty output excluded).
std::tuple<int, int, int, int, int> group_class(gbpoly_precision prec, const gbpoly_gemm_desc* descs, int count) {
  std::vector<int64_t> m, n, k;
  for(int i = 0; i < count; ++i) {
    if(descs[i].M <= 0 || descs[i].N <= 0) continue;
    m.push_back(descs[i].M), n.push_back(descs[i].N), k.push_back(std::max<int64_t>(descs[i].K, 1));
  }
  auto median = [](std::vector<int64_t>& v) -> int64_t {
    if(v.empty()) return 0;
    std::nth_element(v.begin(), v.begin() + v.size() / 2, v.end());
    return v[v.size() / 2];
  };
  return std::make_tuple(int(prec), ceil_log2(int64_t(m.size())), ceil_log2(median(m)), ceil_log2(median(n)),
      ceil_log2(median(k)));
}

}  // namespace gbpoly

using namespace gbpoly;

extern "C" {

gbpoly_status gbpoly_gemm_config_count(gbpoly_precision prec, int* count) {
  if(!count) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *count = tensor_config_count(prec);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_gemm_config_set(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K,
    int config) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  if(config < 0 || config >= tensor_config_count(prec)) return fail(GBPOLY_ERR_INVALID, "no such tile configuration");
  ctx->tuned[shape_bucket(prec, M, N, K)] = config;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_gemm_config_get(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K,
    int* config) {
  if(!ctx || !config) return fail(GBPOLY_ERR_INVALID, "bad argument");
  *config = tuned_config(ctx, prec, M, N, K);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_autotune_gemm(gbpoly_ctx* ctx, gbpoly_precision prec, int64_t M, int64_t N, int64_t K, int reps,
    int* best_config, float* best_ms) {
  if(!ctx) return fail(GBPOLY_ERR_INVALID, "null context");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  const int nconf = tensor_config_count(prec);
  if(nconf == 0) return fail(GBPOLY_ERR_UNSUPPORTED, "form has no tile configurations to tune");
  if(M <= 0 || N <= 0 || K <= 0 || reps <= 0) return fail(GBPOLY_ERR_INVALID, "bad shape or repetition count");
  float *A = nullptr, *B = nullptr, *C = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  gbpoly_status st = GBPOLY_OK;
  int best = 0;
  float best_t = INFINITY;
  auto cleanup = [&] {
    if(A) cudaFree(A);
    if(B) cudaFree(B);
    if(C) cudaFree(C);
    if(e0) cudaEventDestroy(e0);
    if(e1) cudaEventDestroy(e1);
  };
  cudaError_t e = cudaMalloc(&A, size_t(M) * K * 4);
  if(e == cudaSuccess) e = cudaMalloc(&B, size_t(K) * N * 4);
  if(e == cudaSuccess) e = cudaMalloc(&C, size_t(M) * N * 4);
  if(e == cudaSuccess) e = cudaEventCreate(&e0);
  if(e == cudaSuccess) e = cudaEventCreate(&e1);
  if(e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "autotune buffers");
  }
  fill_kernel<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(A, M * K, 1u);
  fill_kernel<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(B, K * N, 2u);
  GemmF32Args a{};
  a.M = M, a.N = N, a.K = K, a.alpha = 1.f, a.beta = 0.f, a.op_a = GBPOLY_OP_N, a.op_b = GBPOLY_OP_N;
  a.A = A, a.lda = K, a.B = B, a.ldb = N, a.C = C, a.ldc = N;
  for(int c = 0; c < nconf && st == GBPOLY_OK; ++c) {
    if((st = launch_gemm_tensor_config(ctx, prec, c, a)) != GBPOLY_OK) break;  // warm-up
    cudaEventRecord(e0, ctx->stream);
    for(int r = 0; r < reps && st == GBPOLY_OK; ++r) st = launch_gemm_tensor_config(ctx, prec, c, a);
    cudaEventRecord(e1, ctx->stream);
    if((e = cudaEventSynchronize(e1)) != cudaSuccess) {
      st = cuda_fail(e, "autotune timing");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= reps;
    if(ms < best_t) {
      best_t = ms;
      best = c;
    }
  }
  cleanup();
  if(st != GBPOLY_OK) return st;
  ctx->tuned[shape_bucket(prec, M, N, K)] = best;
  if(best_config) *best_config = best;
  if(best_ms) *best_ms = best_t;
  return gbpoly_synchronize(ctx);
}

gbpoly_status gbpoly_grouped_config_count(gbpoly_precision prec, int* count) {
  if(!count) return fail(GBPOLY_ERR_INVALID, "null output pointer");
  *count = grouped_config_count(prec);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_grouped_config_set(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int config) {
  if(!ctx || count < 0 || (count > 0 && !descs)) return fail(GBPOLY_ERR_INVALID, "bad argument");
  if(config < 0 || config >= grouped_config_count(prec))
    return fail(GBPOLY_ERR_INVALID, "no such grouped tile configuration");
  ctx->tuned_grouped[group_class(prec, descs, count)] = config;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_grouped_config_get(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int* config) {
  if(!ctx || !config || count < 0 || (count > 0 && !descs)) return fail(GBPOLY_ERR_INVALID, "bad argument");
  *config = default_grouped_config(ctx, prec, descs, count);
  return GBPOLY_OK;
}

gbpoly_status gbpoly_autotune_grouped(gbpoly_ctx* ctx, gbpoly_precision prec, const gbpoly_gemm_desc* descs,
    int count, int reps, int* best_config, float* best_ms) {
  if(!ctx || count <= 0 || !descs || reps <= 0) return fail(GBPOLY_ERR_INVALID, "bad argument");
  GBPOLY_CUDA_TRY(cudaSetDevice(ctx->device));
  const int nconf = grouped_config_count(prec);
  if(nconf == 0) return fail(GBPOLY_ERR_UNSUPPORTED, "form has no grouped tile configurations to tune");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if(e == cudaSuccess) e = cudaEventCreate(&e1);
  if(e != cudaSuccess) {
    if(e0) cudaEventDestroy(e0);
    return cuda_fail(e, "autotune events");
  }
  gbpoly_status st = GBPOLY_OK;
  int best = 0;
  float best_t = INFINITY;
  for(int c = 0; c < nconf && st == GBPOLY_OK; ++c) {
    gbpoly_grouped* g = nullptr;
    if((st = grouped_plan_config(ctx, prec, descs, count, c, &g)) != GBPOLY_OK) break;
    st = gbpoly_grouped_run(ctx, g);  // warm-up
    if(st == GBPOLY_OK) {
      cudaEventRecord(e0, ctx->stream);
      for(int r = 0; r < reps && st == GBPOLY_OK; ++r) st = gbpoly_grouped_run(ctx, g);
      cudaEventRecord(e1, ctx->stream);
      if(st == GBPOLY_OK && (e = cudaEventSynchronize(e1)) != cudaSuccess) st = cuda_fail(e, "autotune timing");
    }
    float ms = 0.f;
    if(st == GBPOLY_OK) cudaEventElapsedTime(&ms, e0, e1);
    gbpoly_status st2 = gbpoly_grouped_destroy(ctx, g);
    if(st == GBPOLY_OK) st = st2;
    if(st == GBPOLY_OK && (st = gbpoly_synchronize(ctx)) == GBPOLY_OK && ms / reps < best_t) {
      best_t = ms / reps;
      best = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if(st != GBPOLY_OK) return st;
  ctx->tuned_grouped[group_class(prec, descs, count)] = best;
  if(best_config) *best_config = best;
  if(best_ms) *best_ms = best_t;
  return GBPOLY_OK;
}

gbpoly_status gbpoly_autotune_save(gbpoly_ctx* ctx, const char* path) {
  if(!ctx || !path) return fail(GBPOLY_ERR_INVALID, "bad argument");
  // keep other devices' entries, replace this device's
  std::vector<std::string> keep;
  const std::string me = device_key(ctx);
  {
    std::ifstream in(path);
    std::string line;
    while(std::getline(in, line))
      if(!line.empty() && line.rfind(me + "\t", 0) != 0) keep.push_back(line);
  }
  std::ofstream out(path, std::ios::trunc);
  if(!out) return fail(GBPOLY_ERR_INVALID, std::string("cannot write ") + path);
  for(auto& l : keep) out << l << "\n";
  for(auto& kv : ctx->tuned)
    out << me << "\t" << std::get<0>(kv.first) << "\t" << std::get<1>(kv.first) << "\t" << std::get<2>(kv.first)
        << "\t" << std::get<3>(kv.first) << "\t" << kv.second << "\n";
  // grouped plans: "G", then form, log2 buckets of count, median M, N, K, configuration
  for(auto& kv : ctx->tuned_grouped)
    out << me << "\tG\t" << std::get<0>(kv.first) << "\t" << std::get<1>(kv.first) << "\t"
        << std::get<2>(kv.first) << "\t" << std::get<3>(kv.first) << "\t" << std::get<4>(kv.first) << "\t"
        << kv.second << "\n";
  return out.good() ? GBPOLY_OK : fail(GBPOLY_ERR_INVALID, std::string("write failed: ") + path);
}

gbpoly_status gbpoly_autotune_load(gbpoly_ctx* ctx, const char* path, int* loaded) {
  if(!ctx || !path) return fail(GBPOLY_ERR_INVALID, "bad argument");
  std::ifstream in(path);
  if(!in) return fail(GBPOLY_ERR_INVALID, std::string("cannot read ") + path);
  const std::string me = device_key(ctx);
  std::string line;
  int n = 0;
  while(std::getline(in, line)) {
    if(line.rfind(me + "\t", 0) != 0) continue;
    if(line.compare(me.size() + 1, 2, "G\t") == 0) {
      std::istringstream f(line.substr(me.size() + 3));
      int prec, cb, bm, bn, bk, config;
      if(!(f >> prec >> cb >> bm >> bn >> bk >> config)) continue;
      if(config < 0 || config >= grouped_config_count(gbpoly_precision(prec))) continue;
      ctx->tuned_grouped[std::make_tuple(prec, cb, bm, bn, bk)] = config;
      ++n;
      continue;
    }
    std::istringstream f(line.substr(me.size() + 1));
    int prec, bm, bn, bk, config;
    if(!(f >> prec >> bm >> bn >> bk >> config)) continue;
    if(config < 0 || config >= tensor_config_count(gbpoly_precision(prec))) continue;
    ctx->tuned[std::make_tuple(prec, bm, bn, bk)] = config;
    ++n;
  }
  if(loaded) *loaded = n;
  return GBPOLY_OK;
}

}  // extern "C"
