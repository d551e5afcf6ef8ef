// Conjugate gradients with the diagonal preconditioner that allocates no
// device memory.  For callers that must not allocate while they run, such
// as a JVM or host framework that has already reserved its GPU memory, or
// a real-time loop that forbids allocation.
//
// All workspace lives in one file-scope static device array.  The CUDA
// driver reserves it when it loads the library's module on a device (with
// the default lazy module loading: at the first call on that device), and
// that device holds it until the process exits.  Host code must not use the
// array's name as a device address (on the host it names a shadow, not
// device memory), so the first call on each device looks up the device
// address with cudaGetSymbolAddress and caches it.  A cudaDeviceReset
// unloads the module and makes the cached address stale: after a reset of
// a device, this entry point must not be called on it again in the same
// process.
//
// The kernels compute exactly what rsg_solver_solve computes for CG with the
// diagonal preconditioner (mtj/src/no/uib/cipr/matrix/sparse/CG.java:58-87,
// DiagonalPreconditioner.java:44-78), including the reduction order, so the
// two entry points give the same iterates.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace {

constexpr int RT = 256;
constexpr int MAX_BLOCKS = 16384;
constexpr int HIST_CAP = 4096;
constexpr size_t VEC_BYTES = (size_t)RSG_NOALLOC_MAX_ROWS * sizeof(double);

struct NState {
  double rho, rho_1, beta, alpha, residual, initR, rtol, atol, dtol;
  int iter, maxIter, status, first, hist_len;
};

// scratch layout: r | z | p | q | invdiag | partials (2 x MAX_BLOCKS) | NState | ticket | history
constexpr size_t OFF_PART = 5 * VEC_BYTES;
constexpr size_t OFF_STATE = OFF_PART + 2 * MAX_BLOCKS * sizeof(double);
constexpr size_t OFF_TICKET = OFF_STATE + 256;
constexpr size_t OFF_HIST = OFF_TICKET + 256;
constexpr size_t SCRATCH_BYTES = OFF_HIST + HIST_CAP * sizeof(double);

static __device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

std::mutex g_mu;
void* g_addr[64] = {};

__device__ __forceinline__ double jmax(double a, double b) { return (a != a || b != b) ? NAN : (a >= b ? a : b); }

__device__ int n_monitor(NState* s, double r, double* hist) {
  if (s->hist_len < HIST_CAP) hist[s->hist_len] = r;
  s->hist_len++;
  s->residual = r;
  if (s->iter == 0) s->initR = r;
  if (r < jmax(s->rtol * s->initR, s->atol)) return 1;
  if (r > s->dtol * s->initR) return -RSG_NOT_CONVERGED_DIVERGENCE;
  if (s->iter >= s->maxIter) return -RSG_NOT_CONVERGED_ITERATIONS;
  if (r != r) return -RSG_NOT_CONVERGED_DIVERGENCE;
  return 0;
}

enum { E_TOP = 1, E_RHO, E_ALPHA, E_NEXT };

__device__ void n_epilogue(int epi, NState* s, double t, double* hist) {
  switch (epi) {
    case E_TOP: {
      // a zero diagonal found by k_n_init stays the call's status even when
      // the initial residual already meets the tolerance
      int m = n_monitor(s, sqrt(t), hist);
      if (m != 0) atomicCAS(&s->status, 0, m);
      break;
    }
    case E_RHO:
      s->rho = t;
      if (!s->first) s->beta = s->rho / s->rho_1;
      break;
    case E_ALPHA: s->alpha = s->rho / t; break;
    case E_NEXT: {
      s->rho_1 = s->rho;
      s->iter++;
      s->first = 0;
      int m = n_monitor(s, sqrt(t), hist);
      if (m != 0) atomicCAS(&s->status, 0, m);
      break;
    }
  }
}

struct Scr {
  double *r, *z, *p, *q, *inv, *part, *hist;
  NState* s;
  unsigned* ticket;
};

__device__ void n_reduce(double v, Scr w, int epi) {
  __shared__ double sh[RT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) sh[wp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0;
    for (int i = 0; i < RT / 32; ++i) x += sh[i];
    w.part[blockIdx.x] = x;
    __threadfence();
    unsigned t = atomicAdd(w.ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double x = 0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) x += __ldcg(w.part + b);
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  __syncthreads();
  if (lane == 0) sh[wp] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double y = 0;
    for (int i = 0; i < RT / 32; ++i) y += sh[i];
    *w.ticket = 0;
    n_epilogue(epi, w.s, y, w.hist);
  }
}

__device__ __forceinline__ bool n_stopped(const NState* s) { return *(volatile const int*)&s->status != 0; }

__device__ __forceinline__ double row_dot(const int* rp, const int* col, const double* val, const double* x, int row) {
  double d = 0;
  for (int q = rp[row]; q < rp[row + 1]; ++q) d += val[q] * x[col[q]];
  return d;
}

// r = b + (-1) A x; reduces r.r; also builds 1/diag (zero diagonal -> status)
__global__ void __launch_bounds__(RT) k_n_init(int n, const int* rp, const int* col, const double* val,
                                               const double* x, const double* b, Scr w) {
  double acc = 0;
  for (int row = blockIdx.x * RT + threadIdx.x; row < n; row += gridDim.x * RT) {
    double ri = b[row] + -1.0 * row_dot(rp, col, val, x, row);
    w.r[row] = ri;
    acc += ri * ri;
    double d = 0;
    for (int q = rp[row]; q < rp[row + 1]; ++q)
      if (col[q] == row) d = val[q];
    if (d == 0) atomicCAS(&w.s->status, 0, -RSG_ZERO_PIVOT);
    w.inv[row] = 1 / d;
  }
  n_reduce(acc, w, E_TOP);
}

// z = r .* invdiag; reduces r.z
__global__ void __launch_bounds__(RT) k_n_precond_dot(int n, Scr w) {
  if (n_stopped(w.s)) return;
  double acc = 0;
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    double zi = w.r[i] * w.inv[i];
    w.z[i] = zi;
    acc += w.r[i] * zi;
  }
  n_reduce(acc, w, E_RHO);
}

__global__ void k_n_p(int n, Scr w) {
  if (n_stopped(w.s)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (w.s->first) w.p[i] = w.z[i];
  else {
    double pi = w.p[i] * w.s->beta;
    w.p[i] = pi + w.z[i];
  }
}

// q = A p (mult semantics); reduces p.q
__global__ void __launch_bounds__(RT) k_n_spmv_dot(int n, const int* rp, const int* col, const double* val, Scr w) {
  if (n_stopped(w.s)) return;
  double acc = 0;
  for (int row = blockIdx.x * RT + threadIdx.x; row < n; row += gridDim.x * RT) {
    double d = row_dot(rp, col, val, w.p, row);
    double qi = (d != 0) ? d : 0.0;
    w.q[row] = qi;
    acc += w.p[row] * qi;
  }
  n_reduce(acc, w, E_ALPHA);
}

// x += alpha p; r += -alpha q; reduces r.r
__global__ void __launch_bounds__(RT) k_n_update(int n, double* x, Scr w) {
  if (n_stopped(w.s)) return;
  const double alpha = w.s->alpha, ma = -alpha;
  double acc = 0;
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    if (alpha != 0) x[i] += alpha * w.p[i];
    double ri = w.r[i];
    if (ma != 0) ri += ma * w.q[i];
    w.r[i] = ri;
    acc += ri * ri;
  }
  n_reduce(acc, w, E_NEXT);
}

// Launches one kernel and returns that launch's own error, leaving any
// error the caller's thread recorded before this call untouched.
template <typename... KArgs, typename... Args>
cudaError_t launch(void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.stream = st;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace

extern "C" rsg_status rsg_cg_diagonal_noalloc(int32_t device, void* stream, int32_t n, int32_t nnz,
                                              const int32_t* d_row_ptr, const int32_t* d_col, const double* d_val,
                                              const double* d_b, double* d_x, double rtol, double atol, double dtol,
                                              int32_t max_iter, rsg_solve_info* info) {
  if (n <= 0 || n > RSG_NOALLOC_MAX_ROWS) return RSG_BAD_ARG;  // rows beyond the static workspace
  if (nnz < 0 || !d_row_ptr || !d_col || !d_val || !d_b || !d_x || max_iter < 0 || device < 0 || device >= 64)
    return RSG_BAD_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return RSG_CUDA_ERROR;
  if (cudaSetDevice(device) != cudaSuccess) return RSG_CUDA_ERROR;
  rsg_status status = RSG_OK;
  do {
    void* base = nullptr;
    {
      // one-time set-up per device: device address of the static workspace
      std::lock_guard<std::mutex> lk(g_mu);
      if (!g_addr[device]) {
        void* a = nullptr;
        if (cudaGetSymbolAddress(&a, g_scratch) != cudaSuccess || !a) {
          status = RSG_CUDA_ERROR;
          break;
        }
        g_addr[device] = a;
      }
      base = g_addr[device];
    }
    unsigned char* b8 = (unsigned char*)base;
    Scr w;
    w.r = (double*)(b8);
    w.z = (double*)(b8 + VEC_BYTES);
    w.p = (double*)(b8 + 2 * VEC_BYTES);
    w.q = (double*)(b8 + 3 * VEC_BYTES);
    w.inv = (double*)(b8 + 4 * VEC_BYTES);
    w.part = (double*)(b8 + OFF_PART);
    w.s = (NState*)(b8 + OFF_STATE);
    w.ticket = (unsigned*)(b8 + OFF_TICKET);
    w.hist = (double*)(b8 + OFF_HIST);
    // the workspace keeps the previous call's contents: reset the state and
    // the reduction ticket before the first kernel
    NState hs = {};
    hs.rho_1 = hs.beta = hs.alpha = 1;
    hs.rtol = rtol;
    hs.atol = atol;
    hs.dtol = dtol;
    hs.maxIter = max_iter;
    hs.first = 1;
    if (cudaMemcpyAsync(w.s, &hs, sizeof(hs), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(w.ticket, 0, sizeof(unsigned), st) != cudaSuccess) {
      status = RSG_CUDA_ERROR;
      break;
    }
    const int nblk = std::max(1, std::min((n + RT - 1) / RT, MAX_BLOCKS));
    const int eb = (n + 255) / 256;
    if (launch(k_n_init, nblk, RT, st, n, d_row_ptr, d_col, d_val, (const double*)d_x, d_b, w) != cudaSuccess) {
      status = RSG_CUDA_ERROR;
      break;
    }
    for (int guard = 0; guard <= max_iter + 1; ++guard) {
      if (cudaMemcpyAsync(&hs, w.s, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        status = RSG_CUDA_ERROR;
        break;
      }
      if (hs.status != 0) break;
      if (launch(k_n_precond_dot, nblk, RT, st, n, w) != cudaSuccess || launch(k_n_p, eb, 256, st, n, w) != cudaSuccess ||
          launch(k_n_spmv_dot, nblk, RT, st, n, d_row_ptr, d_col, d_val, w) != cudaSuccess ||
          launch(k_n_update, nblk, RT, st, n, d_x, w) != cudaSuccess) {
        status = RSG_CUDA_ERROR;
        break;
      }
    }
    if (status != RSG_OK) break;
    if (info) {
      info->iterations = hs.iter;
      info->residual = hs.residual;
      info->initial_residual = hs.initR;
      info->inner_iterations = 0;
      info->refinements = 0;
      info->reason = hs.status < 0 ? -hs.status : RSG_OK;
    }
    if (hs.status < 0) status = -hs.status;
  } while (false);
  cudaSetDevice(prev);
  return status;
}
