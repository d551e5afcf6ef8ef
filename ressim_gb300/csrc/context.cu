// Context management and profiling entry points of the C ABI.
#include <algorithm>

#include "common.cuh"

namespace rsg {

cudaEvent_t Context::get_event() {
  if (!event_pool.empty()) {
    cudaEvent_t e = event_pool.back();
    event_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  RSG_CUDA(cudaEventCreate(&e));
  return e;
}

void Context::flush_profile() {
  for (auto& p : pending) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      auto& e = profile[p.name];
      e.ms += ms;
      e.launches += 1;
    }
    event_pool.push_back(p.a);
    event_pool.push_back(p.b);
  }
  pending.clear();
}

void Context::sync() {
  RSG_CUDA(cudaStreamSynchronize(stream));
  if (profiling) flush_profile();
}

void Context::check_device_error() {
  int* h = static_cast<int*>(pinned) + 512;  // upper half of the staging page
  RSG_CUDA(cudaMemcpyAsync(h, dev_err.get(), sizeof(int), cudaMemcpyDeviceToHost, stream));
  sync();
  if (*h != 0) {
    const int at = *h;
    RSG_CUDA(cudaMemsetAsync(dev_err.get(), 0, sizeof(int), stream));
    sync();
    throw Error(RSG_TIMEOUT, "a level walk's wait ran out at level " + std::to_string(at - 1));
  }
}

}  // namespace rsg

using rsg::guarded;

extern "C" {

int32_t rsg_abi_version(void) { return RSG_ABI_VERSION; }

const char* rsg_status_string(rsg_status s) {
  switch (s) {
    case RSG_OK: return "OK";
    case RSG_NOT_CONVERGED_ITERATIONS: return "NOT_CONVERGED_ITERATIONS";
    case RSG_NOT_CONVERGED_DIVERGENCE: return "NOT_CONVERGED_DIVERGENCE";
    case RSG_NOT_CONVERGED_BREAKDOWN: return "NOT_CONVERGED_BREAKDOWN";
    case RSG_ZERO_PIVOT: return "ZERO_PIVOT";
    case RSG_MISSING_DIAGONAL: return "MISSING_DIAGONAL";
    case RSG_OUT_OF_PATTERN: return "OUT_OF_PATTERN";
    case RSG_NONPOSITIVE_PRESSURE: return "NONPOSITIVE_PRESSURE";
    case RSG_NEGATIVE_MOLES: return "NEGATIVE_MOLES";
    case RSG_BAD_ARG: return "BAD_ARG";
    case RSG_CUDA_ERROR: return "CUDA_ERROR";
    case RSG_TIMEOUT: return "TIMEOUT";
    case RSG_UNSUPPORTED: return "UNSUPPORTED";
    case RSG_NEWTON_NOT_CONVERGED: return "NEWTON_NOT_CONVERGED";
    case RSG_SINGULAR: return "SINGULAR";
    case RSG_PHYSICS: return "PHYSICS";
  }
  return "UNKNOWN";
}

rsg_status rsg_context_create(int32_t device, rsg_ctx** out) {
  if (!out) return RSG_BAD_ARG;
  *out = nullptr;
  rsg_ctx* h = new rsg_ctx();
  rsg_status st = guarded(&h->c, [&] {
    int count = 0;
    RSG_CUDA(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) throw rsg::Error(RSG_CUDA_ERROR, "no such CUDA device");
    cudaDeviceProp prop;
    RSG_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) throw rsg::Error(RSG_CUDA_ERROR, "resgpu needs a Blackwell (sm_10x) GPU");
    RSG_CUDA(cudaSetDevice(device));
    h->c.device = device;
    h->c.num_sms = prop.multiProcessorCount;
    RSG_CUDA(cudaStreamCreateWithFlags(&h->c.stream, cudaStreamNonBlocking));
    RSG_CUDA(cudaMallocHost(&h->c.pinned, 4096));
    h->c.dev_err.resize(1);
    RSG_CUDA(cudaMemsetAsync(h->c.dev_err.get(), 0, sizeof(int), h->c.stream));
  });
  if (st != RSG_OK) {
    delete h;
    return st;
  }
  *out = h;
  return RSG_OK;
}

rsg_status rsg_context_destroy(rsg_ctx* ctx) {
  if (!ctx) return RSG_BAD_ARG;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  for (auto& p : ctx->c.pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : ctx->c.event_pool) cudaEventDestroy(e);
  for (auto e : ctx->c.timers)
    if (e) cudaEventDestroy(e);
  if (ctx->c.pinned) cudaFreeHost(ctx->c.pinned);
  if (ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
  delete ctx;
  return RSG_OK;
}

const char* rsg_context_last_error(rsg_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }

int64_t rsg_context_kernel_launches(rsg_ctx* ctx) { return ctx ? ctx->c.launches : 0; }

rsg_status rsg_context_synchronize(rsg_ctx* ctx) {
  if (!ctx) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] { ctx->c.sync(); });
}

rsg_status rsg_context_set_profiling(rsg_ctx* ctx, int32_t enabled) {
  if (!ctx) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] {
    ctx->c.sync();
    ctx->c.profiling = enabled != 0;
  });
}

rsg_status rsg_context_profile_reset(rsg_ctx* ctx) {
  if (!ctx) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] {
    ctx->c.sync();
    ctx->c.profile.clear();
  });
}

rsg_status rsg_context_profile_read(rsg_ctx* ctx, int32_t max_entries, double* ms, int64_t* launches, char* names,
                                    int32_t names_len, int32_t* n_entries) {
  if (!ctx) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] {
    ctx->c.sync();
    std::string all;
    int k = 0;
    for (auto& kv : ctx->c.profile) {
      if (k >= max_entries) break;
      if (ms) ms[k] = kv.second.ms;
      if (launches) launches[k] = kv.second.launches;
      all += kv.first;
      all += "\n";
      k++;
    }
    if (names && names_len > 0) {
      size_t len = std::min((size_t)names_len - 1, all.size());
      std::memcpy(names, all.data(), len);
      names[len] = 0;
    }
    if (n_entries) *n_entries = k;
  });
}

rsg_status rsg_context_timer_record(rsg_ctx* ctx, int32_t slot) {
  if (!ctx || slot < 0 || slot >= 64) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] {
    auto& t = ctx->c.timers;
    if (!t[slot]) RSG_CUDA(cudaEventCreate(&t[slot]));
    RSG_CUDA(cudaEventRecord(t[slot], ctx->c.stream));
  });
}

rsg_status rsg_context_timer_elapsed(rsg_ctx* ctx, int32_t a, int32_t b, double* ms) {
  if (!ctx || !ms || a < 0 || a >= 64 || b < 0 || b >= 64) return RSG_BAD_ARG;
  return guarded(&ctx->c, [&] {
    auto& t = ctx->c.timers;
    if (!t[a] || !t[b]) throw rsg::Error(RSG_BAD_ARG, "timer slot not recorded");
    RSG_CUDA(cudaEventSynchronize(t[b]));
    float f = 0;
    RSG_CUDA(cudaEventElapsedTime(&f, t[a], t[b]));
    *ms = f;
  });
}

rsg_status rsg_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return RSG_BAD_ARG;
  *ptr = nullptr;
  if (cudaMallocHost(ptr, bytes ? bytes : 1) != cudaSuccess) return RSG_CUDA_ERROR;
  return RSG_OK;
}

rsg_status rsg_host_free(void* ptr) {
  if (ptr) cudaFreeHost(ptr);
  return RSG_OK;
}

}  // extern "C"
