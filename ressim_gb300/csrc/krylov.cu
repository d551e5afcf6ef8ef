// Krylov drivers: CG (mtj/src/no/uib/cipr/matrix/sparse/CG.java:58-87),
// BiCGstab (sparse/BiCGstab.java:65-116) and restarted GMRES
// (sparse/GMRES.java:127-176), with DefaultIterationMonitor semantics
// (sparse/DefaultIterationMonitor.java:132-156).
//
// Scalars live on the device (KState).  Every reduction is a fused kernel
// whose last block reduces the per-block partial sums in a fixed order (the
// result is run-to-run deterministic) and then evaluates the scalar step of
// the algorithm (monitor test, alpha, omega, Givens rotations...).  Kernels
// after a terminating test see KState.status != 0 and return at once, so the
// host only reads the state between batches of iterations.
#include <algorithm>
#include <cmath>

#include "linalg.cuh"

namespace rsg {

void launch_spmv_add(Context& ctx, Csr& A, double alpha, const double* x, double* y, const int* active);
void set_ssor_params(Precond* p, double wf, double wr, int reverse);
void release_trans_plan(const Precond* p);

namespace {

constexpr int RT = 256;  // threads of reduction kernels

enum Epi {
  EPI_NONE = 0,
  EPI_BICG_TOP,    // monitor(|r|), rho_1 = rtilde.r, breakdown checks
  EPI_BICG_ALPHA,  // alpha = rho_1 / (rtilde.v)
  EPI_BICG_S,      // monitor(|s|)
  EPI_BICG_OMEGA,  // omega = (t.s)/(t.t)
  EPI_BICG_NEXT,   // rho_2 = rho_1; iter++; then as TOP
  EPI_CG_TOP,      // monitor(|r|)
  EPI_CG_RHO,      // rho = r.z, beta
  EPI_CG_ALPHA,    // alpha = rho / (p.q)
  EPI_CG_NEXT,     // rho_1 = rho; iter++; monitor(|r|)
  EPI_BICG_S_IN,   // inner (mixed precision) s check against the initial residual of the inner solve
  EPI_GM_NORMR,    // normr = |r| (no monitor)
  EPI_GM_OUTER,    // iter++ (unless first); monitor(normr); inner setup + monitor(|s0|)
  EPI_GM_H,        // H(k,i) = w.v_k
  EPI_GM_NORMW,    // H(i+1,i) = |w|, rotations, i++, iter++, inner monitor
};

// Java's Math.max propagates NaN.
__device__ __forceinline__ double jmax(double a, double b) { return (a != a || b != b) ? NAN : (a >= b ? a : b); }

// DefaultIterationMonitor.convergedI; returns 1 converged, 0 continue,
// negative status on failure.
__device__ int monitor(KState* s, double r, double* hist) {
  if (s->hist_len < s->hist_cap) hist[s->hist_len] = r;
  s->hist_len++;
  s->residual = r;
  if (s->iter == 0) s->initR = r;
  if (r < jmax(s->rtol * s->initR, s->atol)) return 1;
  if (r > s->dtol * s->initR) return -RSG_NOT_CONVERGED_DIVERGENCE;
  if (s->iter >= s->maxIter) return -RSG_NOT_CONVERGED_ITERATIONS;
  if (r != r) return -RSG_NOT_CONVERGED_DIVERGENCE;
  return 0;
}

struct GmresDev {
  double* H;   // (restart+1) x restart, column major
  double* sv;  // restart+1
  double* gc;  // rotation cosines
  double* gs;  // rotation sines
};

__device__ void bicg_top(KState* s, double rr, double rtr, double* hist) {
  int m = monitor(s, sqrt(rr), hist);
  if (m != 0) {
    s->status = m;
    return;
  }
  s->rho_1 = rtr;
  if (s->rho_1 == 0) {
    s->status = -RSG_NOT_CONVERGED_BREAKDOWN;
    return;
  }
  if (s->omega == 0) {
    s->status = -RSG_NOT_CONVERGED_BREAKDOWN;
    return;
  }
  if (!s->first) s->beta = (s->rho_1 / s->rho_2) * (s->alpha / s->omega);
}

// GivensRotation(x, y) (mtj/src/no/uib/cipr/matrix/GivensRotation.java:42-58)
__device__ void givens(double x, double y, double* c, double* sn) {
  double roe = fabs(x) > fabs(y) ? x : y;
  double scale = fabs(x) + fabs(y);
  if (scale != 0) {
    double xs = x / scale, ys = y / scale;
    double r = scale * sqrt(xs * xs + ys * ys);
    if (roe < 0) r *= -1;
    *c = x / r;
    *sn = y / r;
  } else {
    *c = 1;
    *sn = 0;
  }
}

__device__ void run_epilogue(int epi, KState* s, const double* t, double* hist, GmresDev g, int k) {
  switch (epi) {
    case EPI_BICG_TOP: bicg_top(s, t[0], t[1], hist); break;
    case EPI_BICG_ALPHA: s->alpha = s->rho_1 / t[0]; break;
    case EPI_BICG_S: {
      int m = monitor(s, sqrt(t[0]), hist);
      if (m == 1) s->status = KS_CONVERGED_S;
      else if (m < 0) s->status = m;
      break;
    }
    case EPI_BICG_S_IN:
      // unlike BiCGstab.java's check, the initial residual is not replaced
      // by |s| on the first iteration, so an exact preconditioner converges
      if (sqrt(t[0]) < jmax(s->rtol * s->initR, s->atol)) s->status = KS_CONVERGED_S;
      break;
    case EPI_BICG_OMEGA: s->omega = t[0] / t[1]; break;
    case EPI_BICG_NEXT:
      s->rho_2 = s->rho_1;
      s->iter++;
      s->first = 0;
      bicg_top(s, t[0], t[1], hist);
      break;
    case EPI_CG_TOP: {
      int m = monitor(s, sqrt(t[0]), hist);
      if (m != 0) s->status = m;
      break;
    }
    case EPI_CG_RHO:
      s->rho = t[0];
      if (!s->first) s->beta = s->rho / s->rho_1;
      break;
    case EPI_CG_ALPHA: s->alpha = s->rho / t[0]; break;
    case EPI_CG_NEXT: {
      s->rho_1 = s->rho;
      s->iter++;
      s->first = 0;
      int m = monitor(s, sqrt(t[0]), hist);
      if (m != 0) s->status = m;
      break;
    }
    case EPI_GM_NORMR: s->rho = sqrt(t[0]); break;  // normr kept in rho
    case EPI_GM_OUTER: {
      // outer loop test; iter.next() of the outer loop happened already
      int m = monitor(s, sqrt(t[0]), hist);
      if (m != 0) {
        s->status = m;
        break;
      }
      s->rho = sqrt(t[0]);
      // v[0].set(1/normr, r); s.zero().set(0, normr); i = 0
      s->vscale = 1 / s->rho;
      for (int q = 0; q <= s->restart; ++q) g.sv[q] = 0;
      g.sv[0] = s->rho;
      s->gm_i = 0;
      s->gm_exit = 0;
      m = monitor(s, fabs(g.sv[0]), hist);
      if (m == 1) s->gm_exit = 1;
      else if (m < 0) s->status = m;
      break;
    }
    case EPI_GM_H: {
      const int i = s->gm_i, ld = s->restart + 1;
      g.H[k + i * ld] = t[0];
      break;
    }
    case EPI_GM_NORMW: {
      const int i = s->gm_i, ld = s->restart + 1;
      double* H = g.H;
      H[i + 1 + i * ld] = sqrt(t[0]);
      s->vscale = 1. / H[i + 1 + i * ld];
      for (int q = 0; q < i; ++q) {
        double a = H[q + i * ld], b = H[q + 1 + i * ld];
        double temp = g.gc[q] * a + g.gs[q] * b;
        H[q + 1 + i * ld] = -g.gs[q] * a + g.gc[q] * b;
        H[q + i * ld] = temp;
      }
      givens(H[i + i * ld], H[i + 1 + i * ld], &g.gc[i], &g.gs[i]);
      {
        double a = H[i + i * ld], b = H[i + 1 + i * ld];
        double temp = g.gc[i] * a + g.gs[i] * b;
        H[i + 1 + i * ld] = -g.gs[i] * a + g.gc[i] * b;
        H[i + i * ld] = temp;
      }
      {
        double a = g.sv[i], b = g.sv[i + 1];
        double temp = g.gc[i] * a + g.gs[i] * b;
        g.sv[i + 1] = -g.gs[i] * a + g.gc[i] * b;
        g.sv[i] = temp;
      }
      s->gm_i = i + 1;
      s->iter++;
      if (s->gm_i < s->restart) {
        int m = monitor(s, fabs(g.sv[s->gm_i]), hist);
        if (m == 1) s->gm_exit = 1;
        else if (m < 0) s->status = m;
      } else
        s->gm_exit = 1;
      break;
    }
  }
}

// Block-wide deterministic sum of K values, then last-block finish.
template <int K>
__device__ void reduce_finish(double (&v)[K], double* part, unsigned* ticket, int epi, KState* s, double* hist,
                              GmresDev g, int k) {
  __shared__ double sh[K][RT / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[q][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < K; ++q) {
      double x = 0;
      for (int i = 0; i < RT / 32; ++i) x += sh[q][i];
      part[q * gridDim.x + blockIdx.x] = x;
    }
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double tot[K];
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += RT) x += __ldcg(part + q * gridDim.x + b);
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    __syncthreads();
    if (lane == 0) sh[q][w] = x;
    __syncthreads();
    double y = 0;
    for (int i = 0; i < RT / 32; ++i) y += sh[q][i];
    tot[q] = y;
  }
  if (threadIdx.x == 0) {
    *ticket = 0;
    run_epilogue(epi, s, tot, hist, g, k);
  }
}

struct RedArgs {
  double* part;
  unsigned* ticket;
  KState* s;
  double* hist;
  GmresDev g;
};

__device__ __forceinline__ bool stopped(const KState* s) { return *(volatile const int*)&s->status != 0; }

// r = b + (-1) A x (r.set(b); A.multAdd(-1, x, r)), optionally rt = r;
// reduces r.r and r.rt.
__global__ void __launch_bounds__(RT) k_resid(int n, const int* __restrict__ sb, const int* __restrict__ rl,
                                              const int* __restrict__ col, const double* __restrict__ val,
                                              const double* __restrict__ x, const double* __restrict__ b,
                                              double* __restrict__ r, double* __restrict__ rt, RedArgs ra, int epi) {
  double v[2] = {0, 0};
  for (int row = blockIdx.x * RT + threadIdx.x; row < n; row += gridDim.x * RT) {
    int base = sb[row >> 5] + (row & 31);
    int len = rl[row];
    double d = 0;
    for (int k = 0; k < len; ++k) {
      int q = base + 32 * k;
      d += val[q] * x[col[q]];
    }
    double ri = b[row] + -1.0 * d;
    r[row] = ri;
    if (rt) rt[row] = ri;
    v[0] += ri * ri;
    v[1] += ri * ri;
  }
  if (epi == EPI_NONE) return;
  reduce_finish<2>(v, ra.part, ra.ticket, epi, ra.s, ra.hist, ra.g, 0);
}

// y = A x (mult semantics) and dots y.w (and y.z, y.y).  Each product is
// fused into its running sum (one rounding per term): on this part the FP64
// pipe, not HBM, bounds an unfused SpMV (a multiply and an add per entry).
// The Krylov iterates therefore differ from MTJ's in the last bits, within
// the solver parity bound; rsg_csr_mult keeps MTJ's unfused arithmetic.
template <int K>
__global__ void __launch_bounds__(RT, 8) k_spmv_dot(int n, const int* __restrict__ sb, const int* __restrict__ rl,
                                                 const int* __restrict__ col, const double* __restrict__ val,
                                                 const double* __restrict__ x, double* __restrict__ y,
                                                 const double* __restrict__ w, RedArgs ra, int epi) {
  if (stopped(ra.s)) return;
  double v[K];
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = 0;
  for (int row = blockIdx.x * RT + threadIdx.x; row < n; row += gridDim.x * RT) {
    int base = sb[row >> 5] + (row & 31);
    int len = rl[row];
    double d = 0;
#pragma unroll 8
    for (int k = 0; k < len; ++k) {
      int q = base + 32 * k;
      d = __fma_rn(val[q], __ldg(x + col[q]), d);
    }
    double yi = (d != 0) ? d : 0.0;
    y[row] = yi;
    if (K == 1) v[0] = __fma_rn(w[row], yi, v[0]);  // rtilde.dot(v) / p.dot(q)
    if (K == 2) {
      v[0] = __fma_rn(yi, w[row], v[0]);  // t.dot(s)
      v[1] = __fma_rn(yi, yi, v[1]);      // t.dot(t)
    }
  }
  reduce_finish<K>(v, ra.part, ra.ticket, epi, ra.s, ra.hist, ra.g, 0);
}

// Generic dot a.b
__global__ void __launch_bounds__(RT) k_dot(int n, const double* __restrict__ a, const double* __restrict__ b,
                                            RedArgs ra, int epi, int k) {
  if (stopped(ra.s)) return;
  double v[1] = {0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) v[0] += a[i] * b[i];
  reduce_finish<1>(v, ra.part, ra.ticket, epi, ra.s, ra.hist, ra.g, k);
}

// ---- BiCGstab elementwise steps
__global__ void k_bicg_p(int n, const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ p,
                         const KState* s) {
  if (stopped(s)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (s->first) {
    p[i] = r[i];
    return;
  }
  // temp.set(-omega, v).add(p); p.set(r).add(beta, temp)
  double mo = -s->omega;
  double temp = (mo == 0) ? 0.0 : mo * v[i];
  temp += p[i];
  double beta = s->beta;
  p[i] = (beta == 0) ? r[i] : r[i] + beta * temp;
}

// s = r - alpha v (s.set(r).add(-alpha, v)), reduces s.s
__global__ void __launch_bounds__(RT) k_bicg_s(int n, const double* __restrict__ r, const double* __restrict__ v,
                                               double* __restrict__ sv, RedArgs ra) {
  if (stopped(ra.s)) return;
  const double ma = -ra.s->alpha;
  double acc[1] = {0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    double si = (ma == 0) ? r[i] : r[i] + ma * v[i];
    sv[i] = si;
    acc[0] += si * si;
  }
  reduce_finish<1>(acc, ra.part, ra.ticket, EPI_BICG_S, ra.s, ra.hist, ra.g, 0);
}

// early exit on |s|: x.add(alpha, phat)
__global__ void k_bicg_xfinal(int n, const double* __restrict__ phat, double* __restrict__ x, KState* s) {
  if (*(volatile int*)&s->status != KS_CONVERGED_S) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a = s->alpha;
  if (i < n && a != 0) x[i] += a * phat[i];
}

__global__ void k_status_fix(KState* s) {
  if (s->status == KS_CONVERGED_S) s->status = KS_CONVERGED;
}

// x += alpha phat; x += omega shat; r = s - omega t; reduces r.r, rtilde.r
__global__ void __launch_bounds__(RT) k_bicg_update(int n, const double* __restrict__ phat,
                                                    const double* __restrict__ shat, const double* __restrict__ sv,
                                                    const double* __restrict__ t, const double* __restrict__ rtilde,
                                                    double* __restrict__ x, double* __restrict__ r, RedArgs ra) {
  if (stopped(ra.s)) return;
  const double alpha = ra.s->alpha, omega = ra.s->omega, mo = -omega;
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    double xi = x[i];
    if (alpha != 0) xi += alpha * phat[i];
    if (omega != 0) xi += omega * shat[i];
    x[i] = xi;
    double ri = (mo == 0) ? sv[i] : sv[i] + mo * t[i];
    r[i] = ri;
    acc[0] += ri * ri;
    acc[1] += rtilde[i] * ri;
  }
  reduce_finish<2>(acc, ra.part, ra.ticket, EPI_BICG_NEXT, ra.s, ra.hist, ra.g, 0);
}

// ---- CG elementwise steps
__global__ void k_cg_p(int n, const double* __restrict__ z, double* __restrict__ p, const KState* s) {
  if (stopped(s)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (s->first) p[i] = z[i];
  else {
    double pi = p[i] * s->beta;
    p[i] = pi + z[i];
  }
}

// x += alpha p; r += -alpha q; reduces r.r
__global__ void __launch_bounds__(RT) k_cg_update(int n, const double* __restrict__ p, const double* __restrict__ q,
                                                  double* __restrict__ x, double* __restrict__ r, RedArgs ra) {
  if (stopped(ra.s)) return;
  const double alpha = ra.s->alpha, ma = -alpha;
  double acc[1] = {0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    if (alpha != 0) x[i] += alpha * p[i];
    double ri = r[i];
    if (ma != 0) ri += ma * q[i];
    r[i] = ri;
    acc[0] += ri * ri;
  }
  reduce_finish<1>(acc, ra.part, ra.ticket, EPI_CG_NEXT, ra.s, ra.hist, ra.g, 0);
}

// ---- GMRES steps
// w += -H(k-1,i) v_{k-1} (when k > 0), then reduce w.v_k (k <= i) or w.w (k = i+1)
__global__ void __launch_bounds__(RT) k_gm_mgs(int n, double* __restrict__ w, const double* __restrict__ vprev,
                                               const double* __restrict__ vk, RedArgs ra, int k, int epi) {
  if (stopped(ra.s)) return;
  const int i = ra.s->gm_i, ld = ra.s->restart + 1;
  const double h = (k > 0) ? -ra.g.H[(k - 1) + i * ld] : 0.0;
  double acc[1] = {0};
  for (int e = blockIdx.x * RT + threadIdx.x; e < n; e += gridDim.x * RT) {
    double we = w[e];
    if (k > 0 && h != 0) {
      we += h * vprev[e];
      w[e] = we;
    }
    acc[0] += (vk ? we * vk[e] : we * we);
  }
  reduce_finish<1>(acc, ra.part, ra.ticket, epi, ra.s, ra.hist, ra.g, k);
}

// y.set(alpha, x) with alpha = KState.vscale
__global__ void k_gm_vset(int n, const double* __restrict__ w, double* __restrict__ v, const KState* s) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = s->vscale;
  v[i] = (a == 0) ? 0.0 : a * w[i];
}

// UpperTriangDenseMatrix(H, i).solve(s, s) -> dtrtrs; then x += s_j v_j
__global__ void k_gm_trisolve(KState* s, GmresDev g) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (s->status < 0) return;
  const int m = s->gm_i, ld = s->restart + 1;
  for (int q = 0; q < m; ++q)
    if (g.H[q + q * ld] == 0) {
      s->status = -RSG_SINGULAR;
      return;
    }
  for (int k = m - 1; k >= 0; --k)
    if (g.sv[k] != 0) {
      g.sv[k] = g.sv[k] / g.H[k + k * ld];
      for (int q = 0; q < k; ++q) g.sv[q] -= g.sv[k] * g.H[q + k * ld];
    }
}

__global__ void k_gm_xupdate(int n, double* __restrict__ x, const double* __restrict__ V, int64_t ldv,
                             const KState* s, GmresDev g) {
  if (s->status < 0) return;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double xe = x[e];
  for (int j = 0; j < s->gm_i; ++j) {
    double sj = g.sv[j];
    if (sj != 0) xe += sj * V[(int64_t)j * ldv + e];
  }
  x[e] = xe;
}

__global__ void k_iter_inc(KState* s) { s->iter++; }

// ---- FP32 inner BiCGstab for the mixed-precision solver.  Vectors and the
// preconditioner are FP32; dot products accumulate in FP64 and the scalar
// recurrences (KState) stay FP64.
__global__ void k_inner_reset(KState* s, double rtol, double atol, int maxIter) {
  KState z = {};
  z.rho_1 = z.rho_2 = z.alpha = z.beta = z.omega = 1;
  z.rtol = rtol;
  z.atol = atol;
  z.dtol = 1e300;
  z.maxIter = maxIter;
  z.first = 1;
  z.hist_cap = 0;
  *s = z;
}

// r = rt = (float) v (x0 = 0), x = 0; reduces r.r twice (rtilde.r = r.r)
__global__ void __launch_bounds__(RT) k_f32_init(int n, const double* __restrict__ v, float* __restrict__ r,
                                                 float* __restrict__ rt, float* __restrict__ x, RedArgs ra) {
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    float ri = (float)v[i];
    r[i] = ri;
    rt[i] = ri;
    x[i] = 0.f;
    acc[0] += (double)ri * ri;
    acc[1] += (double)ri * ri;
  }
  reduce_finish<2>(acc, ra.part, ra.ticket, EPI_BICG_TOP, ra.s, ra.hist, ra.g, 0);
}

__global__ void k_f32_bicg_p(int n, const float* __restrict__ r, const float* __restrict__ v, float* __restrict__ p,
                             const KState* s) {
  if (stopped(s)) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (s->first) {
    p[i] = r[i];
    return;
  }
  const float mo = (float)(-s->omega), beta = (float)s->beta;
  float temp = mo * v[i] + p[i];
  p[i] = r[i] + beta * temp;
}

template <int K>
__global__ void __launch_bounds__(RT, 8) k_f32_spmv_dot(int n, const int* __restrict__ sb, const int* __restrict__ rl,
                                                     const int* __restrict__ col, const float* __restrict__ val,
                                                     const float* __restrict__ x, float* __restrict__ y,
                                                     const float* __restrict__ w, RedArgs ra, int epi) {
  if (stopped(ra.s)) return;
  double v[K];
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = 0;
  for (int row = blockIdx.x * RT + threadIdx.x; row < n; row += gridDim.x * RT) {
    int base = sb[row >> 5] + (row & 31);
    int len = rl[row];
    float d = 0;
#pragma unroll 8
    for (int k = 0; k < len; ++k) {
      int q = base + 32 * k;
      d = fmaf(val[q], __ldg(x + col[q]), d);
    }
    y[row] = d;
    if (K == 1) v[0] += (double)w[row] * d;
    if (K == 2) {
      v[0] += (double)d * w[row];
      v[1] += (double)d * d;
    }
  }
  reduce_finish<K>(v, ra.part, ra.ticket, epi, ra.s, ra.hist, ra.g, 0);
}

__global__ void __launch_bounds__(RT) k_f32_bicg_s(int n, const float* __restrict__ r, const float* __restrict__ v,
                                                   float* __restrict__ sv, RedArgs ra) {
  if (stopped(ra.s)) return;
  const float ma = (float)(-ra.s->alpha);
  double acc[1] = {0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    float si = r[i] + ma * v[i];
    sv[i] = si;
    acc[0] += (double)si * si;
  }
  reduce_finish<1>(acc, ra.part, ra.ticket, EPI_BICG_S_IN, ra.s, ra.hist, ra.g, 0);
}

__global__ void k_f32_bicg_xfinal(int n, const float* __restrict__ phat, float* __restrict__ x, KState* s) {
  if (*(volatile int*)&s->status != KS_CONVERGED_S) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += (float)s->alpha * phat[i];
}

__global__ void __launch_bounds__(RT) k_f32_bicg_update(int n, const float* __restrict__ phat,
                                                        const float* __restrict__ shat, const float* __restrict__ sv,
                                                        const float* __restrict__ t, const float* __restrict__ rtilde,
                                                        float* __restrict__ x, float* __restrict__ r, RedArgs ra) {
  if (stopped(ra.s)) return;
  const float alpha = (float)ra.s->alpha, omega = (float)ra.s->omega;
  double acc[2] = {0, 0};
  for (int i = blockIdx.x * RT + threadIdx.x; i < n; i += gridDim.x * RT) {
    x[i] = x[i] + alpha * phat[i] + omega * shat[i];
    float ri = sv[i] - omega * t[i];
    r[i] = ri;
    acc[0] += (double)ri * ri;
    acc[1] += (double)rtilde[i] * ri;
  }
  reduce_finish<2>(acc, ra.part, ra.ticket, EPI_BICG_NEXT, ra.s, ra.hist, ra.g, 0);
}

__global__ void k_f32_to_f64(int n, const float* __restrict__ a, double* __restrict__ b, const KState* sin,
                             KState* sout) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
  if (i == 0) sout->inner += sin->iter;
}

}  // namespace

// ----------------------------------------------------------------------
struct Solver {
  Context* ctx;
  int method, pc_kind;
  std::unique_ptr<Precond> pc;
  double rtol = 1e-5, atol = 1e-50, dtol = 1e5;
  int maxIter = 100000, restart = 30;
  int n = 0;
  DeviceBuffer<double> w1, w2, w3, w4, w5, w6, w7, w8, w9, V;
  DeviceBuffer<double> part, hist, gmH, gmS, gmC, gmSn;
  DeviceBuffer<unsigned> ticket;
  DeviceBuffer<KState> state;
  // mixed precision: FP32 inner BiCGstab workspace, inner state, Z basis
  int inner_iters = 10;
  double inner_rtol = 1e-3;
  DeviceBuffer<float> f1, f2, f3, f4, f5, f6, f7, f8, fx;
  DeviceBuffer<double> Zb, part_in, hist_in;
  DeviceBuffer<unsigned> ticket_in;
  DeviceBuffer<KState> state_in;
  KState* hstate = nullptr;  // pinned mirror
  int nblk = 0;
  Csr* setup_for = nullptr;

  Solver(Context* c, int m, int p) : ctx(c), method(m), pc_kind(p) {
    pc = make_precond(c, p);
    RSG_CUDA(cudaMallocHost(&hstate, sizeof(KState)));
    state.resize(1);
    ticket.resize(1);
    RSG_CUDA(cudaMemsetAsync(ticket.get(), 0, sizeof(unsigned), ctx->stream));
  }
  ~Solver() {
    if (hstate) cudaFreeHost(hstate);
    release_trans_plan(pc.get());
  }

  void ensure(int n_) {
    if (n_ == n && w1.size()) return;
    n = n_;
    // zero like MTJ's new DenseVector(n): SSOR starts its sweeps from the
    // previous contents of its output vector
    for (auto* b : {&w1, &w2, &w3, &w4, &w5, &w6, &w7, &w8, &w9}) {
      b->resize(n);
      RSG_CUDA(cudaMemsetAsync(b->get(), 0, sizeof(double) * n, ctx->stream));
    }
    nblk = std::max(1, std::min(blocks_for(n, RT), 16384));
    part.resize((size_t)4 * nblk);
  }

  RedArgs red() {
    GmresDev g{gmH.get(), gmS.get(), gmC.get(), gmSn.get()};
    return RedArgs{part.get(), ticket.get(), state.get(), hist.get(), g};
  }

  void init_state() {
    KState s = {};
    s.rho_1 = s.rho_2 = s.alpha = s.beta = s.omega = 1;
    s.rtol = rtol;
    s.atol = atol;
    s.dtol = dtol;
    s.maxIter = maxIter;
    s.first = 1;
    s.restart = restart;
    s.hist_cap = (int)hist.size();
    *hstate = s;
    RSG_CUDA(cudaMemcpyAsync(state.get(), hstate, sizeof(KState), cudaMemcpyHostToDevice, ctx->stream));
  }

  void read_state() {
    RSG_CUDA(cudaMemcpyAsync(hstate, state.get(), sizeof(KState), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
  }

  void solve(Csr& A, const double* b, double* x, rsg_solve_info* info) {
    if (setup_for != &A) throw Error(RSG_BAD_ARG, "rsg_solver_setup must be called with this matrix first");
    ensure(A.n);
    size_t cap = std::min<size_t>((size_t)maxIter * 2 + 64, (size_t)1 << 22);
    if (hist.size() < cap) hist.resize(cap);
    A.refresh_sell();
    init_state();
    switch (method) {
      case RSG_CG: run_cg(A, b, x); break;
      case RSG_BICGSTAB: run_bicgstab(A, b, x); break;
      case RSG_GMRES: run_gmres(A, b, x); break;
      case RSG_FGMRES_MIXED: run_fgmres_mixed(A, b, x); break;
      default: throw Error(RSG_UNSUPPORTED, "unknown iterative method");
    }
    read_state();
    ctx->check_device_error();
    if (info) {
      info->iterations = hstate->iter;
      info->residual = hstate->residual;
      info->initial_residual = hstate->initR;
      info->inner_iterations = hstate->inner;
      info->refinements = 0;
      info->reason = hstate->status < 0 ? -hstate->status : RSG_OK;
    }
    if (hstate->status < 0) {
      int st = -hstate->status;
      char buf[160];
      snprintf(buf, sizeof buf, "%s after %d iterations, residual %.6e", rsg_status_string(st), hstate->iter,
               hstate->residual);
      throw Error(st, buf);
    }
  }

  int batch() const { return 4; }

  void run_bicgstab(Csr& A, const double* b, double* x) {
    // r, rtilde, p, v, phat, s, shat, t
    double *r = w1.get(), *rt = w2.get(), *p = w3.get(), *v = w4.get(), *ph = w5.get(), *s = w6.get(),
           *sh = w7.get(), *t = w8.get();
    int* act = &state.get()->status;
    RSG_LAUNCH(*ctx, "bicg_init", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
               A.sell_val.get(), x, b, r, rt, red(), (int)EPI_BICG_TOP);
    const int eb = blocks_for(n, 256);
    for (;;) {
      read_state();
      if (hstate->status != 0) break;
      for (int it = 0; it < batch(); ++it) {
        RSG_LAUNCH(*ctx, "bicg_p", k_bicg_p, eb, 256, 0, n, r, v, p, state.get());
        pc->apply(p, ph, act);
        RSG_LAUNCH(*ctx, "spmv_dot", k_spmv_dot<1>, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(),
                   A.sell_col.get(), A.sell_val.get(), ph, v, rt, red(), (int)EPI_BICG_ALPHA);
        RSG_LAUNCH(*ctx, "bicg_s", k_bicg_s, nblk, RT, 0, n, r, v, s, red());
        RSG_LAUNCH(*ctx, "bicg_xfinal", k_bicg_xfinal, eb, 256, 0, n, ph, x, state.get());
        RSG_LAUNCH(*ctx, "status_fix", k_status_fix, 1, 1, 0, state.get());
        pc->apply(s, sh, act);
        RSG_LAUNCH(*ctx, "spmv_dot", k_spmv_dot<2>, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(),
                   A.sell_col.get(), A.sell_val.get(), sh, t, s, red(), (int)EPI_BICG_OMEGA);
        RSG_LAUNCH(*ctx, "bicg_update", k_bicg_update, nblk, RT, 0, n, ph, sh, s, t, rt, x, r, red());
      }
    }
  }

  void run_cg(Csr& A, const double* b, double* x) {
    double *r = w1.get(), *z = w2.get(), *p = w3.get(), *q = w4.get();
    int* act = &state.get()->status;
    RSG_LAUNCH(*ctx, "cg_init", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
               A.sell_val.get(), x, b, r, (double*)nullptr, red(), (int)EPI_CG_TOP);
    const int eb = blocks_for(n, 256);
    for (;;) {
      read_state();
      if (hstate->status != 0) break;
      for (int it = 0; it < batch(); ++it) {
        pc->apply(r, z, act);
        RSG_LAUNCH(*ctx, "dot", k_dot, nblk, RT, 0, n, r, z, red(), (int)EPI_CG_RHO, 0);
        RSG_LAUNCH(*ctx, "cg_p", k_cg_p, eb, 256, 0, n, z, p, state.get());
        RSG_LAUNCH(*ctx, "spmv_dot", k_spmv_dot<1>, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(),
                   A.sell_col.get(), A.sell_val.get(), p, q, p, red(), (int)EPI_CG_ALPHA);
        RSG_LAUNCH(*ctx, "cg_update", k_cg_update, nblk, RT, 0, n, p, q, x, r, red());
      }
    }
  }

  // Flexible GMRES(m) in FP64 (right preconditioned, modified Gram-Schmidt,
  // Givens rotations as in GMRES.java) whose preconditioner is a short FP32
  // BiCGstab with the FP32 ILU(0) factors and an FP32 SpMV.  The outer
  // monitor sees the true FP64 residual ||b - A x|| at each restart and the
  // rotated residual estimate inside a cycle, with DefaultIterationMonitor
  // semantics.
  void run_fgmres_mixed(Csr& A, const double* b, double* x) {
    const int m = restart;
    const size_t ld = (size_t)n;
    if (V.size() < (size_t)(m + 1) * ld) V.resize((size_t)(m + 1) * ld);
    if (Zb.size() < (size_t)m * ld) Zb.resize((size_t)m * ld);
    for (auto* f : {&f1, &f2, &f3, &f4, &f5, &f6, &f7, &f8, &fx})
      if (f->size() != (size_t)n) f->resize(n);
    gmH.resize((size_t)(m + 1) * m);
    gmS.resize(m + 1);
    gmC.resize(m + 1);
    gmSn.resize(m + 1);
    part_in.resize((size_t)4 * nblk);
    hist_in.resize(1);
    ticket_in.resize(1);
    state_in.resize(1);
    RSG_CUDA(cudaMemsetAsync(ticket_in.get(), 0, sizeof(unsigned), ctx->stream));
    RSG_CUDA(cudaMemsetAsync(gmH.get(), 0, sizeof(double) * (m + 1) * m, ctx->stream));
    A.refresh_sell_f32();
    double *w = w1.get(), *r = w3.get();
    auto vcol = [&](int j) { return V.get() + (size_t)j * ld; };
    auto zcol = [&](int j) { return Zb.get() + (size_t)j * ld; };
    const int eb = blocks_for(n, 256);
    GmresDev gd{gmH.get(), gmS.get(), gmC.get(), gmSn.get()};
    RedArgs ri{part_in.get(), ticket_in.get(), state_in.get(), hist_in.get(), gd};
    KState* sin = state_in.get();
    const int* act_in = &sin->status;
    float *ir = f1.get(), *irt = f2.get(), *ip = f3.get(), *iv = f4.get(), *iph = f5.get(), *is = f6.get(),
          *ish = f7.get(), *it = f8.get(), *ix = fx.get();
    // r = b - A x; monitor(|r|)
    RSG_LAUNCH(*ctx, "fgm_resid", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
               A.sell_val.get(), x, b, r, (double*)nullptr, red(), (int)EPI_NONE);
    RSG_LAUNCH(*ctx, "fgm_norm", k_dot, nblk, RT, 0, n, r, r, red(), (int)EPI_GM_OUTER, 0);
    for (;;) {
      read_state();
      if (hstate->status != 0) break;
      RSG_LAUNCH(*ctx, "gm_vset", k_gm_vset, eb, 256, 0, n, r, vcol(0), state.get());
      while (!hstate->gm_exit && hstate->status == 0) {
        const int i = hstate->gm_i;
        // z_i = M(v_i): FP32 BiCGstab + ILU(0) from zero
        RSG_LAUNCH(*ctx, "inner_reset", k_inner_reset, 1, 1, 0, sin, inner_rtol, 0.0, inner_iters);
        RSG_LAUNCH(*ctx, "inner_init", k_f32_init, nblk, RT, 0, n, vcol(i), ir, irt, ix, ri);
        for (int q = 0; q < inner_iters; ++q) {
          RSG_LAUNCH(*ctx, "inner_p", k_f32_bicg_p, eb, 256, 0, n, ir, iv, ip, sin);
          pc->apply_f32(ip, iph, act_in);
          RSG_LAUNCH(*ctx, "inner_spmv_dot", k_f32_spmv_dot<1>, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(),
                     A.sell_col.get(), A.sell_valf.get(), iph, iv, irt, ri, (int)EPI_BICG_ALPHA);
          RSG_LAUNCH(*ctx, "inner_s", k_f32_bicg_s, nblk, RT, 0, n, ir, iv, is, ri);
          RSG_LAUNCH(*ctx, "inner_xfinal", k_f32_bicg_xfinal, eb, 256, 0, n, iph, ix, sin);
          RSG_LAUNCH(*ctx, "status_fix", k_status_fix, 1, 1, 0, sin);
          pc->apply_f32(is, ish, act_in);
          RSG_LAUNCH(*ctx, "inner_spmv_dot", k_f32_spmv_dot<2>, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(),
                     A.sell_col.get(), A.sell_valf.get(), ish, it, is, ri, (int)EPI_BICG_OMEGA);
          RSG_LAUNCH(*ctx, "inner_update", k_f32_bicg_update, nblk, RT, 0, n, iph, ish, is, it, irt, ix, ir, ri);
        }
        RSG_LAUNCH(*ctx, "to_f64", k_f32_to_f64, eb, 256, 0, n, ix, zcol(i), (const KState*)sin, state.get());
        // w = A z_i, then the Arnoldi step of GMRES.java:146-162 on w
        launch_spmv(*ctx, A, zcol(i), w, nullptr);
        for (int k2 = 0; k2 <= i; ++k2)
          RSG_LAUNCH(*ctx, "gm_mgs", k_gm_mgs, nblk, RT, 0, n, w, k2 > 0 ? vcol(k2 - 1) : (const double*)nullptr,
                     vcol(k2), red(), k2, (int)EPI_GM_H);
        RSG_LAUNCH(*ctx, "gm_mgs", k_gm_mgs, nblk, RT, 0, n, w, vcol(i), (const double*)nullptr, red(), i + 1,
                   (int)EPI_GM_NORMW);
        RSG_LAUNCH(*ctx, "gm_vset", k_gm_vset, eb, 256, 0, n, w, vcol(i + 1), state.get());
        read_state();
      }
      if (hstate->status != 0) break;
      RSG_LAUNCH(*ctx, "gm_trisolve", k_gm_trisolve, 1, 1, 0, state.get(), gd);
      RSG_LAUNCH(*ctx, "gm_xupdate", k_gm_xupdate, eb, 256, 0, n, x, Zb.get(), (int64_t)ld, state.get(), gd);
      RSG_LAUNCH(*ctx, "fgm_resid", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
                 A.sell_val.get(), x, b, r, (double*)nullptr, red(), (int)EPI_NONE);
      RSG_LAUNCH(*ctx, "iter_inc", k_iter_inc, 1, 1, 0, state.get());
      RSG_LAUNCH(*ctx, "fgm_norm", k_dot, nblk, RT, 0, n, r, r, red(), (int)EPI_GM_OUTER, 0);
    }
  }

  void run_gmres(Csr& A, const double* b, double* x) {
    const int m = restart;
    const size_t ld = (size_t)n;
    if (V.size() < (size_t)(m + 1) * ld) V.resize((size_t)(m + 1) * ld);
    gmH.resize((size_t)(m + 1) * m);
    gmS.resize(m + 1);
    gmC.resize(m + 1);
    gmSn.resize(m + 1);
    RSG_CUDA(cudaMemsetAsync(gmH.get(), 0, sizeof(double) * (m + 1) * m, ctx->stream));
    double *w = w1.get(), *u = w2.get(), *r = w3.get();
    auto vcol = [&](int j) { return V.get() + (size_t)j * ld; };
    const int eb = blocks_for(n, 256);
    // u = b - A x; r = M u; normr = |r|; u = M b
    RSG_LAUNCH(*ctx, "gm_resid", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
               A.sell_val.get(), x, b, u, (double*)nullptr, red(), (int)EPI_NONE);
    pc->apply(u, r, nullptr);
    RSG_LAUNCH(*ctx, "gm_norm", k_dot, nblk, RT, 0, n, r, r, red(), (int)EPI_GM_OUTER, 0);
    pc->apply(b, u, nullptr);
    for (;;) {
      read_state();
      if (hstate->status != 0) break;
      // v[0] = r / normr
      RSG_LAUNCH(*ctx, "gm_vset", k_gm_vset, eb, 256, 0, n, r, vcol(0), state.get());
      while (!hstate->gm_exit && hstate->status == 0) {
        const int i = hstate->gm_i;
        launch_spmv(*ctx, A, vcol(i), u, nullptr);
        pc->apply(u, w, nullptr);
        for (int k = 0; k <= i; ++k)
          RSG_LAUNCH(*ctx, "gm_mgs", k_gm_mgs, nblk, RT, 0, n, w, k > 0 ? vcol(k - 1) : (const double*)nullptr,
                     vcol(k), red(), k, (int)EPI_GM_H);
        RSG_LAUNCH(*ctx, "gm_mgs", k_gm_mgs, nblk, RT, 0, n, w, vcol(i), (const double*)nullptr, red(), i + 1,
                   (int)EPI_GM_NORMW);
        RSG_LAUNCH(*ctx, "gm_vset", k_gm_vset, eb, 256, 0, n, w, vcol(i + 1), state.get());
        read_state();
      }
      if (hstate->status != 0) break;
      GmresDev g{gmH.get(), gmS.get(), gmC.get(), gmSn.get()};
      RSG_LAUNCH(*ctx, "gm_trisolve", k_gm_trisolve, 1, 1, 0, state.get(), g);
      RSG_LAUNCH(*ctx, "gm_xupdate", k_gm_xupdate, eb, 256, 0, n, x, V.get(), (int64_t)ld, state.get(), g);
      RSG_LAUNCH(*ctx, "gm_resid", k_resid, nblk, RT, 0, n, A.slice_base.get(), A.row_len.get(), A.sell_col.get(),
                 A.sell_val.get(), x, b, u, (double*)nullptr, red(), (int)EPI_NONE);
      pc->apply(u, r, nullptr);
      RSG_LAUNCH(*ctx, "iter_inc", k_iter_inc, 1, 1, 0, state.get());
      RSG_LAUNCH(*ctx, "gm_norm", k_dot, nblk, RT, 0, n, r, r, red(), (int)EPI_GM_OUTER, 0);
    }
  }
};

void SolverDeleter::operator()(Solver* s) const { delete s; }

SolverPtr make_solver(Context* ctx, int method, int precond, double rtol, double atol, double dtol, int maxit,
                      int restart) {
  if (method != RSG_CG && method != RSG_BICGSTAB && method != RSG_GMRES && method != RSG_FGMRES_MIXED)
    throw Error(RSG_UNSUPPORTED, "linear solver not available");
  if (method == RSG_FGMRES_MIXED && precond == RSG_PC_SSOR)
    throw Error(RSG_UNSUPPORTED, "the mixed-precision solver takes ILU, AMG, diagonal or no preconditioning");
  SolverPtr s(new Solver(ctx, method, precond));
  s->rtol = rtol;
  s->atol = atol;
  s->dtol = dtol;
  s->maxIter = maxit;
  s->restart = restart;
  return s;
}

void solver_forget_matrix(Solver& s) { s.setup_for = nullptr; }

void solver_setup(Solver& s, Csr& A) {
  s.pc->setup(A);
  s.setup_for = &A;
}

void solver_solve(Solver& s, Csr& A, const double* b, double* x, rsg_solve_info* info) { s.solve(A, b, x, info); }

SolverView solver_view(Solver& s) {
  return SolverView{s.method, s.pc_kind, s.pc.get(), s.rtol, s.atol, s.dtol, s.maxIter, s.setup_for, s.ctx, s.restart, s.inner_iters, s.inner_rtol};
}

void solver_set_inner(Solver& s, int iterations, double rtol) {
  s.inner_iters = iterations;
  s.inner_rtol = rtol;
}

}  // namespace rsg

using rsg::guarded;

extern "C" {

rsg_status rsg_solver_create(rsg_ctx* ctx, int32_t method, int32_t precond, rsg_solver** out) {
  if (!ctx || !out) return RSG_BAD_ARG;
  *out = nullptr;
  if (method < RSG_CG || method > RSG_FGMRES_MIXED) return RSG_BAD_ARG;
  rsg_solver* h = new rsg_solver();
  rsg_status st = guarded(&ctx->c, [&] {
    if (method == RSG_FGMRES_MIXED && precond == RSG_PC_SSOR)
      throw rsg::Error(RSG_UNSUPPORTED, "the mixed-precision solver takes ILU, AMG, diagonal or no preconditioning");
    h->s.reset(new rsg::Solver(&ctx->c, method, precond));
  });
  if (st != RSG_OK) {
    delete h;
    return st;
  }
  *out = h;
  return RSG_OK;
}

rsg_status rsg_solver_destroy(rsg_solver* s) {
  if (!s) return RSG_BAD_ARG;
  if (s->s) cudaStreamSynchronize(s->s->ctx->stream);
  delete s;
  return RSG_OK;
}

rsg_status rsg_solver_set_monitor(rsg_solver* s, double rtol, double atol, double dtol, int32_t max_iter) {
  if (!s || max_iter < 0) return RSG_BAD_ARG;
  s->s->rtol = rtol;
  s->s->atol = atol;
  s->s->dtol = dtol;
  s->s->maxIter = max_iter;
  return RSG_OK;
}

rsg_status rsg_solver_set_restart(rsg_solver* s, int32_t restart) {
  if (!s || restart <= 0) return RSG_BAD_ARG;
  s->s->restart = restart;
  return RSG_OK;
}

rsg_status rsg_solver_set_inner(rsg_solver* s, int32_t inner_iterations, double inner_rtol) {
  if (!s || inner_iterations <= 0) return RSG_BAD_ARG;
  s->s->inner_iters = inner_iterations;
  s->s->inner_rtol = inner_rtol;
  return RSG_OK;
}

rsg_status rsg_solver_set_ssor(rsg_solver* s, double omega_f, double omega_r, int32_t reverse) {
  if (!s) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { rsg::set_ssor_params(s->s->pc.get(), omega_f, omega_r, reverse); });
}

rsg_status rsg_solver_set_walk_shape(rsg_solver* s, int32_t ctas) {
  if (!s || (ctas != 0 && ctas != 8 && ctas != 16)) return RSG_BAD_ARG;
  return rsg::ilu_walk_shape(s->s->pc.get(), ctas, nullptr) ? RSG_OK : RSG_UNSUPPORTED;
}

rsg_status rsg_solver_walk_shapes(rsg_solver* s, int32_t* shapes) {
  if (!s || !shapes) return RSG_BAD_ARG;
  int v[4] = {0, 0, 0, 0};
  if (!rsg::ilu_walk_shape(s->s->pc.get(), -1, v)) return RSG_UNSUPPORTED;
  for (int q = 0; q < 4; ++q) shapes[q] = v[q];
  return RSG_OK;
}

rsg_status rsg_solver_setup(rsg_solver* s, rsg_csr* A) {
  if (!s || !A) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] {
    s->s->pc->setup(A->m);
    s->s->setup_for = &A->m;
  });
}

rsg_status rsg_solver_solve_device(rsg_solver* s, rsg_csr* A, const double* d_b, double* d_x, rsg_solve_info* info) {
  if (!s || !A || !d_b || !d_x) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { s->s->solve(A->m, d_b, d_x, info); });
}

rsg_status rsg_solver_solve(rsg_solver* s, rsg_csr* A, const double* b, double* x, rsg_solve_info* info) {
  if (!s || !A || !b || !x) return RSG_BAD_ARG;
  rsg::Context* ctx = s->s->ctx;
  rsg::DeviceBuffer<double> db, dx;
  rsg_status st = guarded(ctx, [&] {
    int n = A->m.n;
    db.resize(n);
    dx.resize(n);
    RSG_CUDA(cudaMemcpyAsync(db.get(), b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(dx.get(), x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  });
  if (st != RSG_OK) return st;
  rsg_status solve_st = guarded(ctx, [&] { s->s->solve(A->m, db.get(), dx.get(), info); });
  // MTJ leaves x as it stood when the exception was thrown; copy it back either way
  st = guarded(ctx, [&] {
    RSG_CUDA(cudaMemcpyAsync(x, dx.get(), sizeof(double) * A->m.n, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
  });
  return solve_st != RSG_OK ? solve_st : st;
}

static rsg_status precond_host(rsg_solver* s, const double* b, double* x, bool trans) {
  if (!s || !b || !x || !s->s->setup_for) return RSG_BAD_ARG;
  rsg::Context* ctx = s->s->ctx;
  return guarded(ctx, [&] {
    int n = s->s->setup_for->n;
    rsg::DeviceBuffer<double> db(n), dx(n);
    RSG_CUDA(cudaMemcpyAsync(db.get(), b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(dx.get(), x, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if (trans) s->s->pc->trans_apply(db.get(), dx.get(), nullptr);
    else s->s->pc->apply_exact(db.get(), dx.get());
    RSG_CUDA(cudaMemcpyAsync(x, dx.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    ctx->check_device_error();
  });
}

rsg_status rsg_precond_apply(rsg_solver* s, const double* b, double* x) { return precond_host(s, b, x, false); }
rsg_status rsg_precond_trans_apply(rsg_solver* s, const double* b, double* x) { return precond_host(s, b, x, true); }

rsg_status rsg_solver_amg_levels(rsg_solver* s, int32_t* levels) {
  if (!s || !levels) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { *levels = rsg::amg_levels(s->s->pc.get()); });
}

rsg_status rsg_solver_amg_level(rsg_solver* s, int32_t k, int32_t* sizes, int32_t* rowptr, int32_t* col,
                                double* val, int32_t* pt, int32_t* colptr, int32_t* rowind, double* idata) {
  if (!s) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] {
    int sz[4];
    rsg::amg_level_sizes(s->s->pc.get(), k, sz);
    if (sizes)
      for (int q = 0; q < 4; ++q) sizes[q] = sz[q];
    if (rowptr || col || val || pt || colptr || rowind || idata)
      rsg::amg_level_get(s->s->pc.get(), k, rowptr, col, val, pt, colptr, rowind, idata);
  });
}

rsg_status rsg_solver_history(rsg_solver* s, int32_t max_len, double* out, int32_t* len) {
  if (!s) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] {
    rsg::Solver& S = *s->s;
    S.read_state();
    int L = std::min<int>(S.hstate->hist_len, (int)S.hist.size());
    if (len) *len = L;
    if (out && max_len > 0 && L > 0) {
      RSG_CUDA(cudaMemcpyAsync(out, S.hist.get(), sizeof(double) * std::min(L, max_len), cudaMemcpyDeviceToHost,
                               S.ctx->stream));
      S.ctx->sync();
    }
  });
}

}  // extern "C"
