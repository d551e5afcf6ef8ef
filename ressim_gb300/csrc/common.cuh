// Shared infrastructure of the resgpu library: context, device buffers,
// launch accounting, error propagation across the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/rsg.h"

namespace rsg {

// Thrown inside the library, converted to an rsg_status at the C boundary.
struct Error : std::runtime_error {
  rsg_status status;
  Error(rsg_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define RSG_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      throw ::rsg::Error(RSG_CUDA_ERROR, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
struct DeviceBuffer {
  T* ptr = nullptr;
  size_t count = 0;
  DeviceBuffer() {}
  explicit DeviceBuffer(size_t n) { resize(n); }
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  DeviceBuffer(DeviceBuffer&& o) noexcept : ptr(o.ptr), count(o.count) {
    o.ptr = nullptr;
    o.count = 0;
  }
  DeviceBuffer& operator=(DeviceBuffer&& o) noexcept {
    release();
    ptr = o.ptr;
    count = o.count;
    o.ptr = nullptr;
    o.count = 0;
    return *this;
  }
  ~DeviceBuffer() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    count = 0;
  }
  void resize(size_t n) {
    if (n == count && ptr) return;
    release();
    if (n) RSG_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
    count = n;
  }
  T* get() const { return ptr; }
  size_t size() const { return count; }
};

struct ProfileEntry {
  double ms = 0;
  int64_t launches = 0;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int cluster_size = 8;  // CTAs per cluster of the level-scheduled sweeps
  int64_t launches = 0;
  std::string last_error;
  bool profiling = false;
  struct Pending {
    std::string name;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  std::map<std::string, ProfileEntry> profile;
  // pinned host staging for small scalar reads
  void* pinned = nullptr;
  cudaEvent_t timers[64] = {};
  // set by kernels whose bounded waits ran out (1 + site); read after solves
  DeviceBuffer<int> dev_err;

  cudaEvent_t get_event();
  void flush_profile();  // requires a synchronized stream
  void sync();
  // throws RSG_TIMEOUT (and clears the flag) when a kernel's bounded wait ran out
  void check_device_error();
};

// Launch helper: counts launches and (optionally) brackets them with events.
struct LaunchScope {
  Context& ctx;
  const char* name;
  cudaEvent_t a = nullptr;
  LaunchScope(Context& c, const char* n) : ctx(c), name(n) {
    ctx.launches++;
    if (ctx.profiling) {
      a = ctx.get_event();
      cudaEventRecord(a, ctx.stream);
    }
  }
  ~LaunchScope() {
    if (ctx.profiling) {
      cudaEvent_t b = ctx.get_event();
      cudaEventRecord(b, ctx.stream);
      ctx.pending.push_back({name, a, b});
    }
  }
};

inline void check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw Error(RSG_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

// an empty grid (nothing to do, e.g. a mesh without connections) launches nothing
inline bool grid_empty(int g) { return g <= 0; }
inline bool grid_empty(const dim3& g) { return g.x == 0 || g.y == 0 || g.z == 0; }

#define RSG_LAUNCH(ctx, name, kernel, grid, block, smem, ...)                    \
  do {                                                                           \
    if (::rsg::grid_empty(grid)) break;                                          \
    ::rsg::LaunchScope scope_(ctx, name);                                        \
    kernel<<<(grid), (block), (smem), (ctx).stream>>>(__VA_ARGS__);              \
    ::rsg::check_launch(name);                                                   \
  } while (0)

inline int blocks_for(int64_t n, int threads) { return (int)((n + threads - 1) / threads); }

// Runs f and converts exceptions to a status, recording the message.
template <class F>
rsg_status guarded(Context* ctx, F&& f) {
  try {
    f();
    return RSG_OK;
  } catch (const Error& e) {
    if (ctx) ctx->last_error = e.what();
    return e.status;
  } catch (const std::bad_alloc&) {
    if (ctx) ctx->last_error = "host allocation failed";
    return RSG_CUDA_ERROR;
  } catch (const std::exception& e) {
    if (ctx) ctx->last_error = e.what();
    return RSG_BAD_ARG;
  }
}

}  // namespace rsg

struct rsg_ctx {
  rsg::Context c;
};
