// Persistent ensemble pressure solver: the pressure systems of many
// simulator instances (an ensemble of realisations of uneven sizes) are
// solved in ONE launch.  The grid is as many thread-block clusters as fit on
// the GPU at once; each cluster takes the next instance from a device work
// queue and solves it completely with preconditioned BiCGstab
// (mtj/src/no/uib/cipr/matrix/sparse/BiCGstab.java:65-116) and the ILU(0)
// preconditioner (sparse/ILU.java:54-140), reading the instance's matrix,
// factors, walk schedules and vectors through per-instance offsets (a
// descriptor table).  Nothing returns to the host between iterations.
//
// Inside a cluster (CTAs of 256 threads, one per SM):
// * SpMV, BLAS-1 and the BiCGstab recurrences run over 4,096 virtual
//   threads (virtual thread t owns rows t, t + 4096, ...): one per thread in
//   a 16-CTA cluster, two per thread in an 8-CTA cluster.  Values that other
//   SMs wrote earlier in the launch (the walks' outputs, the vectors the
//   walks read) are loaded from L2 (ld.global.cg), never from a possibly
//   stale L1 line or the read-only cache;
// * dot products reduce per virtual warp, then across the 128 virtual warps
//   through distributed shared memory in a fixed tree, so every CTA holds
//   the same scalars and the result does not depend on the cluster shape
//   (16 or 8 CTAs give identical bits);
// * the ILU(0) triangular solves are the level walks of ring.cuh, walked by
//   the first RING_SLICES / CTAS warps of each CTA (all 8 warps of an 8-CTA
//   cluster, 4 of the 8 in a 16-CTA cluster, whose other warps only help
//   with the streaming phases: a 16-SM cluster with 4 warps per SM keeps too
//   few loads in flight to stream a member's matrix).
// Precision 0 is BiCGstab in FP64 with the FP64 factors.  Precision 1 is the
// mixed-precision solver of krylov.cu's run_fgmres_mixed (FP64 flexible
// GMRES around a short FP32 BiCGstab with the FP32 factors and the FP32
// copy of A) in the same persistent form (k_ens_fgmres).
//
// The scalar recurrences, monitor and zero tests follow BiCGstab.java and
// DefaultIterationMonitor.java as krylov.cu's BiCGstab does; only the
// reduction order of the dot products differs from that solver.
#include <algorithm>
#include <map>
#include <mutex>

#include "ring.cuh"

namespace rsg {

namespace {

struct EnsMember {
  int n;
  const int* sb;  // SELL copy of A (FP64 values)
  const int* rl;
  const int* col;
  const double* val;
  RingArgs gl, gu;  // ILU(0) lower and upper walk schedules
  const double* lval;
  const double* uval;
  const double* udiag;
  const float* lvalf;
  const float* uvalf;
  const float* udiagf;
  const double* b;
  double* x;  // initial guess in, solution out
  double* w;  // FP64 BiCGstab: 9 vectors of n (r, rtilde, p, v, phat, s, shat, t, y);
              // FGMRES: r, w, then V (restart + 1 vectors) and Z (restart vectors)
  float* f;   // FGMRES: the 10 FP32 vectors of the inner BiCGstab and its ILU(0) solves
  const float* valf;  // FP32 SELL values of A (inner SpMV)
  double rtol, atol, dtol;
  int maxIter;
  int restart, inner_iters;
  double inner_rtol;
};

struct EnsResult {
  double residual, initR;
  int iterations, status;
  int inner;  // FGMRES: inner FP32 iterations summed
};

struct EnsArgs {
  int count;
  const EnsMember* mem;
  EnsResult* res;
  int* queue;  // next instance to take
  int* abort;  // set when a level walk's wait ran out
};

__device__ __forceinline__ double jmax2(double a, double b) {
  return (a != a || b != b) ? NAN : (a >= b ? a : b);
}

constexpr int ENS_THREADS = 256;  // threads per CTA, both cluster shapes
constexpr int ENS_VT = 4096;      // virtual threads of the row loops
constexpr int ENS_WPC = ENS_THREADS / 32;

template <int CTAS>
struct EnsShape {
  static constexpr int NT = CTAS * ENS_THREADS;  // threads of the cluster
  static constexpr int VPT = ENS_VT / NT;        // virtual threads per thread
  static_assert(VPT * NT == ENS_VT, "the cluster must tile the virtual threads");
};

// The rows of a member, virtual thread by virtual thread: thread gtid runs
// virtual threads gtid + u * NT (u < VPT), virtual thread vt owns rows vt,
// vt + ENS_VT, ..., visited in that order.  f(u, i) for each row i.
template <int CTAS, typename F>
__device__ __forceinline__ void ens_rows(int n, int gtid, F&& f) {
  for (int i0 = gtid; i0 < n; i0 += ENS_VT)
#pragma unroll
    for (int u = 0; u < EnsShape<CTAS>::VPT; ++u) {
      const int i = i0 + u * EnsShape<CTAS>::NT;
      if (i < n) f(u, i);
    }
}

// Row i of a SELL-32 matrix times x, entries summed in column-slot order
// (FUSED: one rounding per entry, else the product rounded, then the sum);
// x comes from L2 (written by other SMs in the launch).  Unrolled by 8 so
// that the loads of 8 entries can be in flight together.  (Loading 16
// entries into register arrays first made the kernel's register demand
// spill into the level walks it calls, which then ran 2.5x slower.)
template <bool FUSED, typename T>
__device__ __forceinline__ T ens_row(const T* __restrict__ val, const int* __restrict__ col, const T* x, int base,
                                     int len) {
  T d = 0;
#pragma unroll 8
  for (int k = 0; k < len; ++k) {
    const int q = base + 32 * k;
    if constexpr (!FUSED) d += val[q] * __ldcg(x + col[q]);
    else if constexpr (sizeof(T) == 4) d = fmaf(val[q], __ldcg(x + col[q]), d);
    else d = __fma_rn(val[q], __ldcg(x + col[q]), d);
  }
  return d;
}

// Sum over the member's virtual threads of K values each (v[u][q]: virtual
// thread gtid + u * NT); every thread gets the totals.  The lanes of each
// virtual warp (32 consecutive virtual threads, the lanes of one warp) are
// summed first; then lane l of each CTA's warp 0 adds virtual warps
// (l + l+32) + (l+64 + l+96) and the lanes are summed again, the same tree
// for either cluster shape.  part: shared [2][3][VPT * ENS_WPC], tot:
// shared [3]; ph alternates the two halves of part so one barrier per
// reduction suffices.
template <int CTAS, int K>
__device__ __forceinline__ void cluster_sum(double (&v)[EnsShape<CTAS>::VPT][K], double* part, double* tot, int& ph,
                                            cg::cluster_group& cluster) {
  constexpr int VPT = EnsShape<CTAS>::VPT, VW = VPT * ENS_WPC, WARPS = EnsShape<CTAS>::NT / 32;
  static_assert(ENS_VT / 32 == 128, "the fixed tree adds 128 virtual warps");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int u = 0; u < VPT; ++u)
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double x = v[u][q];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) part[(ph * 3 + q) * VW + u * ENS_WPC + w] = x;
    }
  cluster.sync();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      double y[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int vw = lane + 32 * j, u = vw / WARPS, rw = vw % WARPS;
        y[j] = *cluster.map_shared_rank(part + (ph * 3 + q) * VW + u * ENS_WPC + rw % ENS_WPC, rw / ENS_WPC);
      }
      double x = (y[0] + y[1]) + (y[2] + y[3]);
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) tot[q] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int u = 0; u < VPT; ++u)
#pragma unroll
    for (int q = 0; q < K; ++q) v[u][q] = tot[q];
  ph ^= 1;
}

// A walk as a called function: its registers are allocated apart from the
// solver loop's, which keeps both free of spills.  FP64 rows are summed with
// fused multiply-adds, as the stream path's solver applies do.
// (13 entries of a row in registers, as for the 27-point stencil; longer
// rows read the rest from memory)
// The schedule and vectors are copied into local variables first: through
// the caller's references they would live in global memory, and every store
// of the walk would force the compiler to load them again.
template <int KIND, typename T, int CTAS>
__device__ __noinline__ bool walk(const RingArgs& g, const RingVals<T>& a, unsigned char* smem) {
  const RingArgs gl = g;
  const RingVals<T> al = a;
  return ring_walk<KIND, T, 13, CTAS, ENS_THREADS, true>(gl, al, smem);
}

// out = M^-1 in (ILU(0): L y = in, U out = y, FP64 factors) on the cluster;
// ends with a cluster barrier, so out is complete for every thread of the
// cluster.
template <int CTAS>
__device__ __noinline__ bool ens_precond(const EnsMember& m, const double* in, double* out, unsigned char* smem,
                                         cg::cluster_group& cluster) {
  double* y = m.w + 8 * (size_t)m.n;
  const RingVals<double> lo{m.lval, nullptr, in, y, nullptr};
  if (!walk<SW_ILU_LOWER, double, CTAS>(m.gl, lo, smem)) return false;
  const RingVals<double> up{m.uval, m.udiag, y, out, nullptr};
  if (!walk<SW_ILU_UPPER, double, CTAS>(m.gu, up, smem)) return false;
  cluster.sync();
  return true;
}

template <int CTAS>
__global__ void __launch_bounds__(ENS_THREADS) k_ens_bicgstab(EnsArgs e, size_t) {
  constexpr int VPT = EnsShape<CTAS>::VPT;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double part[2 * 3 * VPT * ENS_WPC];
  __shared__ double tot[3];
  __shared__ int take;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int gtid = rank * ENS_THREADS + (int)threadIdx.x;
  int ph = 0;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) take = *(volatile int*)e.abort ? e.count : atomicAdd(e.queue, 1);
    cluster.sync();
    const int mi = *cluster.map_shared_rank(&take, 0);
    cluster.sync();  // CTA 0 rewrites take only after every CTA has read it
    if (mi >= e.count) return;
    const EnsMember m = e.mem[mi];  // a local copy: global stores do not force reloads
    const int n = m.n;
    double *r = m.w, *rt = m.w + (size_t)n, *p = m.w + 2 * (size_t)n, *v = m.w + 3 * (size_t)n;
    double *phat = m.w + 4 * (size_t)n, *s = m.w + 5 * (size_t)n, *shat = m.w + 6 * (size_t)n;
    double *t = m.w + 7 * (size_t)n, *x = m.x;
    const double rtol = m.rtol, atol = m.atol, dtol = m.dtol;
    const int maxIter = m.maxIter;
    double rho_1 = 1, rho_2 = 1, alpha = 1, beta = 1, omega = 1, resid = 0, initR = 0;
    int iter = 0, first = 1, status = KS_RUNNING;
    // DefaultIterationMonitor.convergedI: 1 converged, 0 go on, < 0 failure
    auto monitor = [&](double rn) -> int {
      resid = rn;
      if (iter == 0) initR = rn;
      if (rn < jmax2(rtol * initR, atol)) return 1;
      if (rn > dtol * initR) return -RSG_NOT_CONVERGED_DIVERGENCE;
      if (iter >= maxIter) return -RSG_NOT_CONVERGED_ITERATIONS;
      if (rn != rn) return -RSG_NOT_CONVERGED_DIVERGENCE;
      return 0;
    };
    // top of an iteration: monitor |r|, rho_1 = rtilde.r, breakdown tests, beta
    auto top = [&](double rr, double rtr) {
      const int mo = monitor(sqrt(rr));
      if (mo != 0) {
        status = mo;
        return;
      }
      rho_1 = rtr;
      if (rho_1 == 0 || omega == 0) {
        status = -RSG_NOT_CONVERGED_BREAKDOWN;
        return;
      }
      if (!first) beta = (rho_1 / rho_2) * (alpha / omega);
    };
    bool walked = true;
    {
      // r = b + (-1) A x, rtilde = r (unfused row sums, as A.multAdd)
      double a2[VPT][2] = {};
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        const double d = ens_row<false>(m.val, m.col, x, m.sb[i >> 5] + (i & 31), m.rl[i]);
        const double ri = m.b[i] + -1.0 * d;
        r[i] = ri;
        rt[i] = ri;
        a2[u][0] += ri * ri;
        a2[u][1] += ri * ri;
      });
      cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
      top(a2[0][0], a2[0][1]);
    }
    while (status == KS_RUNNING) {
      // p = r + beta (p - omega v)
      {
        const double mo = -omega, bt = beta;
        const bool fst = first;
        ens_rows<CTAS>(n, gtid, [&](int, int i) {
          if (fst) {
            p[i] = r[i];
            return;
          }
          double temp = (mo == 0) ? 0.0 : mo * v[i];
          temp += p[i];
          p[i] = (bt == 0) ? r[i] : r[i] + bt * temp;
        });
      }
      if (!(walked = ens_precond<CTAS>(m, p, phat, smem, cluster))) break;
      {
        // v = A phat; alpha = rho_1 / (rtilde . v)
        double a1[VPT][1] = {};
        ens_rows<CTAS>(n, gtid, [&](int u, int i) {
          const double d = ens_row<true>(m.val, m.col, (const double*)phat, m.sb[i >> 5] + (i & 31), m.rl[i]);
          const double yi = (d != 0) ? d : 0.0;
          v[i] = yi;
          a1[u][0] = __fma_rn(rt[i], yi, a1[u][0]);
        });
        cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
        alpha = rho_1 / a1[0][0];
      }
      {
        // s = r - alpha v; monitor |s|
        double a1[VPT][1] = {};
        const double ma = -alpha;
        ens_rows<CTAS>(n, gtid, [&](int u, int i) {
          const double si = (ma == 0) ? r[i] : r[i] + ma * v[i];
          s[i] = si;
          a1[u][0] += si * si;
        });
        cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
        const int mo = monitor(sqrt(a1[0][0]));
        if (mo == 1) {
          // x.add(alpha, phat) and stop
          const double al = alpha;
          if (al != 0) ens_rows<CTAS>(n, gtid, [&](int, int i) { x[i] += al * __ldcg(phat + i); });
          status = KS_CONVERGED;
          break;
        }
        if (mo < 0) {
          status = mo;
          break;
        }
      }
      if (!(walked = ens_precond<CTAS>(m, s, shat, smem, cluster))) break;
      {
        // t = A shat; omega = (t . s) / (t . t)
        double a2[VPT][2] = {};
        ens_rows<CTAS>(n, gtid, [&](int u, int i) {
          const double d = ens_row<true>(m.val, m.col, (const double*)shat, m.sb[i >> 5] + (i & 31), m.rl[i]);
          const double yi = (d != 0) ? d : 0.0;
          t[i] = yi;
          a2[u][0] = __fma_rn(yi, s[i], a2[u][0]);
          a2[u][1] = __fma_rn(yi, yi, a2[u][1]);
        });
        cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
        omega = a2[0][0] / a2[0][1];
      }
      {
        // x += alpha phat + omega shat; r = s - omega t; reduce r.r, rtilde.r
        double a2[VPT][2] = {};
        const double al = alpha, om = omega, mo = -omega;
        ens_rows<CTAS>(n, gtid, [&](int u, int i) {
          double xi = x[i];
          if (al != 0) xi += al * __ldcg(phat + i);
          if (om != 0) xi += om * __ldcg(shat + i);
          x[i] = xi;
          const double ri = (mo == 0) ? s[i] : s[i] + mo * t[i];
          r[i] = ri;
          a2[u][0] += ri * ri;
          a2[u][1] += rt[i] * ri;
        });
        cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
        rho_2 = rho_1;
        iter++;
        first = 0;
        top(a2[0][0], a2[0][1]);
      }
    }
    if (!walked) {
      if (gtid == 0) {
        atomicExch(e.abort, 1);
        e.res[mi] = EnsResult{resid, initR, iter, RSG_TIMEOUT, 0};
      }
      return;  // this cluster's shared memory may still receive pushes
    }
    cluster.sync();  // the last updates of x are in place before the next instance
    if (gtid == 0) e.res[mi] = EnsResult{resid, initR, iter, status == KS_CONVERGED ? RSG_OK : -status, 0};
  }
}

// ------------------------------------------------------------ FGMRES ----
// Mixed precision: FP64 flexible GMRES(m) (right preconditioned, modified
// Gram-Schmidt, Givens rotations as GMRES.java:84-176 and krylov.cu's
// run_fgmres_mixed) whose preconditioner is a short FP32 BiCGstab with the
// FP32 ILU(0) factors and the FP32 copy of A.  The outer monitor sees the
// true FP64 residual at each restart and the rotated estimate inside a cycle.
// The Hessenberg matrix, rotations and outer scalars live in each CTA's
// shared memory; thread 0 of every CTA applies each epilogue to its copy
// from the same cluster-wide sums, so the copies stay identical.
struct GmShared {
  double rho, vscale, resid, initR;
  int iter, status, gi, gexit, inner;
};

__device__ __forceinline__ int gm_monitor(GmShared& g, const EnsMember& m, double r) {
  g.resid = r;
  if (g.iter == 0) g.initR = r;
  if (r < jmax2(m.rtol * g.initR, m.atol)) return 1;
  if (r > m.dtol * g.initR) return -RSG_NOT_CONVERGED_DIVERGENCE;
  if (g.iter >= m.maxIter) return -RSG_NOT_CONVERGED_ITERATIONS;
  if (r != r) return -RSG_NOT_CONVERGED_DIVERGENCE;
  return 0;
}

// GivensRotation(x, y) (mtj/src/no/uib/cipr/matrix/GivensRotation.java:42-58)
__device__ __forceinline__ void ens_givens(double x, double y, double* c, double* sn) {
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

// out = M^-1 in with the FP32 factors (L y = in, U out = y)
template <int CTAS>
__device__ __noinline__ bool ens_ilu_f32(const EnsMember& m, const float* in, float* y, float* out,
                                         unsigned char* smem) {
  const RingVals<float> lo{m.lvalf, nullptr, in, y, nullptr};
  if (!walk<SW_ILU_LOWER, float, CTAS>(m.gl, lo, smem)) return false;
  const RingVals<float> up{m.uvalf, m.udiagf, y, out, nullptr};
  return walk<SW_ILU_UPPER, float, CTAS>(m.gu, up, smem);
}

// The FP32 inner BiCGstab from x = 0 on v (krylov.cu k_inner_reset,
// k_f32_*): inner_iters steps at most, inner_rtol against its own initial
// residual, no divergence test; z = its iterate.  Its SpMV fuses each
// product (as k_f32_spmv_dot).  Returns false when a walk timed out.  Every
// thread ends with the same inner iteration count.
template <int CTAS>
__device__ bool ens_inner(const EnsMember& m, const double* v, double* z, unsigned char* smem, double* part,
                          double* tot, int& ph, int gtid, cg::cluster_group& cluster, int& inner_its) {
  constexpr int VPT = EnsShape<CTAS>::VPT;
  const int n = m.n;
  float *ir = m.f, *irt = m.f + (size_t)n, *ip = m.f + 2 * (size_t)n, *iv = m.f + 3 * (size_t)n;
  float *iph = m.f + 4 * (size_t)n, *is = m.f + 5 * (size_t)n, *ish = m.f + 6 * (size_t)n;
  float *it = m.f + 7 * (size_t)n, *ix = m.f + 8 * (size_t)n, *iy = m.f + 9 * (size_t)n;
  double rho_1 = 1, rho_2 = 1, alpha = 1, beta = 1, omega = 1, initR = 0;
  int iter = 0, first = 1, status = KS_RUNNING;
  auto monitor = [&](double rn) -> int {
    if (iter == 0) initR = rn;
    if (rn < jmax2(m.inner_rtol * initR, 0.0)) return 1;
    if (iter >= m.inner_iters) return -RSG_NOT_CONVERGED_ITERATIONS;
    if (rn != rn) return -RSG_NOT_CONVERGED_DIVERGENCE;
    return 0;
  };
  auto top = [&](double rr, double rtr) {
    const int mo = monitor(sqrt(rr));
    if (mo != 0) {
      status = mo;
      return;
    }
    rho_1 = rtr;
    if (rho_1 == 0 || omega == 0) {
      status = -RSG_NOT_CONVERGED_BREAKDOWN;
      return;
    }
    if (!first) beta = (rho_1 / rho_2) * (alpha / omega);
  };
  {
    double a2[VPT][2] = {};
    ens_rows<CTAS>(n, gtid, [&](int u, int i) {
      const float ri = (float)v[i];
      ir[i] = ri;
      irt[i] = ri;
      ix[i] = 0.f;
      a2[u][0] += (double)ri * ri;
      a2[u][1] += (double)ri * ri;
    });
    cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
    top(a2[0][0], a2[0][1]);
  }
  while (status == KS_RUNNING) {
    {
      const float mo = (float)(-omega), bf = (float)beta;
      const bool fst = first;
      ens_rows<CTAS>(n, gtid, [&](int, int i) {
        if (fst) {
          ip[i] = ir[i];
          return;
        }
        const float temp = mo * iv[i] + ip[i];
        ip[i] = ir[i] + bf * temp;
      });
    }
    if (!ens_ilu_f32<CTAS>(m, ip, iy, iph, smem)) return false;
    {
      double a1[VPT][1] = {};
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        const float d = ens_row<true>(m.valf, m.col, (const float*)iph, m.sb[i >> 5] + (i & 31), m.rl[i]);
        iv[i] = d;
        a1[u][0] += (double)irt[i] * d;
      });
      cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
      alpha = rho_1 / a1[0][0];
    }
    {
      double a1[VPT][1] = {};
      const float ma = (float)(-alpha);
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        const float si = ir[i] + ma * iv[i];
        is[i] = si;
        a1[u][0] += (double)si * si;
      });
      cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
      // the inner s check keeps the initial residual (krylov.cu EPI_BICG_S_IN)
      if (sqrt(a1[0][0]) < jmax2(m.inner_rtol * initR, 0.0)) {
        const float af = (float)alpha;
        ens_rows<CTAS>(n, gtid, [&](int, int i) { ix[i] += af * __ldcg(iph + i); });
        status = KS_CONVERGED;
        break;
      }
    }
    if (!ens_ilu_f32<CTAS>(m, is, iy, ish, smem)) return false;
    {
      double a2[VPT][2] = {};
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        const float d = ens_row<true>(m.valf, m.col, (const float*)ish, m.sb[i >> 5] + (i & 31), m.rl[i]);
        it[i] = d;
        a2[u][0] += (double)d * is[i];
        a2[u][1] += (double)d * d;
      });
      cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
      omega = a2[0][0] / a2[0][1];
    }
    {
      double a2[VPT][2] = {};
      const float af = (float)alpha, of = (float)omega;
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        ix[i] = ix[i] + af * __ldcg(iph + i) + of * __ldcg(ish + i);
        const float ri = is[i] - of * it[i];
        ir[i] = ri;
        a2[u][0] += (double)ri * ri;
        a2[u][1] += (double)irt[i] * ri;
      });
      cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
      rho_2 = rho_1;
      iter++;
      first = 0;
      top(a2[0][0], a2[0][1]);
    }
  }
  ens_rows<CTAS>(n, gtid, [&](int, int i) { z[i] = (double)ix[i]; });
  inner_its += iter;
  return true;
}

template <int CTAS>
__global__ void __launch_bounds__(ENS_THREADS) k_ens_fgmres(EnsArgs e, size_t ring_bytes) {
  constexpr int VPT = EnsShape<CTAS>::VPT;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double part[2 * 3 * VPT * ENS_WPC];
  __shared__ double tot[3];
  __shared__ int take;
  __shared__ GmShared g;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int gtid = rank * ENS_THREADS + (int)threadIdx.x;
  const bool lead = threadIdx.x == 0;
  int ph = 0;
  for (;;) {
    if (rank == 0 && lead) take = *(volatile int*)e.abort ? e.count : atomicAdd(e.queue, 1);
    cluster.sync();
    const int mi = *cluster.map_shared_rank(&take, 0);
    cluster.sync();
    if (mi >= e.count) return;
    const EnsMember m = e.mem[mi];  // a local copy: global stores do not force reloads
    const int n = m.n, mr = m.restart, ld = mr + 1;
    double* H = reinterpret_cast<double*>(smem + ring_bytes);  // (m + 1) x m, column major
    double *sv = H + (size_t)ld * mr, *gc = sv + ld, *gs = gc + ld;
    double *r = m.w, *w = m.w + (size_t)n, *V = m.w + 2 * (size_t)n, *Z = V + (size_t)ld * n, *x = m.x;
    if (lead) {
      g.iter = 0;
      g.status = 0;
      g.inner = 0;
      g.initR = g.resid = 0;
      for (int q = 0; q < ld * mr; ++q) H[q] = 0;
    }
    __syncthreads();
    bool walked = true;
    int inner = 0;
    for (;;) {
      // r = b - A x (A.multAdd order: unfused row sums); |r|
      double a1[VPT][1] = {};
      ens_rows<CTAS>(n, gtid, [&](int u, int i) {
        const double d = ens_row<false>(m.val, m.col, (const double*)x, m.sb[i >> 5] + (i & 31), m.rl[i]);
        const double ri = m.b[i] + -1.0 * d;
        r[i] = ri;
        a1[u][0] += ri * ri;
      });
      cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
      if (lead) {
        // outer loop test, then the first inner test on |s_0| = |r|
        int mo = gm_monitor(g, m, sqrt(a1[0][0]));
        if (mo != 0) {
          g.status = mo;
        } else {
          g.rho = sqrt(a1[0][0]);
          g.vscale = 1 / g.rho;
          for (int q = 0; q <= mr; ++q) sv[q] = 0;
          sv[0] = g.rho;
          g.gi = 0;
          g.gexit = 0;
          mo = gm_monitor(g, m, fabs(sv[0]));
          if (mo == 1) g.gexit = 1;
          else if (mo < 0) g.status = mo;
        }
      }
      __syncthreads();
      if (g.status != 0) break;
      {
        const double a = g.vscale;
        ens_rows<CTAS>(n, gtid, [&](int, int i) { V[i] = (a == 0) ? 0.0 : a * r[i]; });
      }
      while (!g.gexit && g.status == 0) {
        const int i = g.gi;
        double* vi = V + (size_t)i * n;
        double* zi = Z + (size_t)i * n;
        // z_i = M(v_i): the inner walks start with a cluster barrier, which publishes v_i
        if (!(walked = ens_inner<CTAS>(m, vi, zi, smem, part, tot, ph, gtid, cluster, inner))) break;
        cluster.sync();  // z_i complete before the SpMV gathers it
        // w = A z_i (mult: unfused row sums, exact zeros stored as +0)
        ens_rows<CTAS>(n, gtid, [&](int, int q) {
          const double d = ens_row<false>(m.val, m.col, (const double*)zi, m.sb[q >> 5] + (q & 31), m.rl[q]);
          w[q] = (d != 0) ? d : 0.0;
        });
        // modified Gram-Schmidt (GMRES.java:146-162), one reduction per basis vector
        for (int k2 = 0; k2 <= i + 1; ++k2) {
          const double h = (k2 > 0) ? -H[(k2 - 1) + i * ld] : 0.0;
          const double* vprev = k2 > 0 ? V + (size_t)(k2 - 1) * n : nullptr;
          const double* vk = k2 <= i ? V + (size_t)k2 * n : nullptr;
          double acc[VPT][1] = {};
          ens_rows<CTAS>(n, gtid, [&](int u, int q) {
            double we = w[q];
            if (k2 > 0 && h != 0) {
              we += h * vprev[q];
              w[q] = we;
            }
            acc[u][0] += vk ? we * vk[q] : we * we;
          });
          cluster_sum<CTAS, 1>(acc, part, tot, ph, cluster);
          if (k2 <= i) {
            if (lead) H[k2 + i * ld] = acc[0][0];
            __syncthreads();
          } else if (lead) {
            // H(i+1,i) = |w|, rotations (krylov.cu EPI_GM_NORMW)
            H[i + 1 + i * ld] = sqrt(acc[0][0]);
            g.vscale = 1. / H[i + 1 + i * ld];
            for (int q = 0; q < i; ++q) {
              const double a = H[q + i * ld], b = H[q + 1 + i * ld];
              const double temp = gc[q] * a + gs[q] * b;
              H[q + 1 + i * ld] = -gs[q] * a + gc[q] * b;
              H[q + i * ld] = temp;
            }
            ens_givens(H[i + i * ld], H[i + 1 + i * ld], &gc[i], &gs[i]);
            {
              const double a = H[i + i * ld], b = H[i + 1 + i * ld];
              const double temp = gc[i] * a + gs[i] * b;
              H[i + 1 + i * ld] = -gs[i] * a + gc[i] * b;
              H[i + i * ld] = temp;
            }
            {
              const double a = sv[i], b = sv[i + 1];
              const double temp = gc[i] * a + gs[i] * b;
              sv[i + 1] = -gs[i] * a + gc[i] * b;
              sv[i] = temp;
            }
            g.gi = i + 1;
            g.iter++;
            if (g.gi < mr) {
              const int mo = gm_monitor(g, m, fabs(sv[g.gi]));
              if (mo == 1) g.gexit = 1;
              else if (mo < 0) g.status = mo;
            } else {
              g.gexit = 1;
            }
          }
        }
        __syncthreads();
        {
          const double a = g.vscale;
          double* vn = V + (size_t)(i + 1) * n;
          ens_rows<CTAS>(n, gtid, [&](int, int q) { vn[q] = (a == 0) ? 0.0 : a * w[q]; });
        }
      }
      if (!walked || g.status != 0) break;
      // UpperTriangDenseMatrix(H, i).solve(s, s), then x += sum_j s_j z_j
      if (lead) {
        const int mm = g.gi;
        bool singular = false;
        for (int q = 0; q < mm; ++q)
          if (H[q + q * ld] == 0) singular = true;
        if (singular) {
          g.status = -RSG_SINGULAR;
        } else {
          for (int k = mm - 1; k >= 0; --k)
            if (sv[k] != 0) {
              sv[k] = sv[k] / H[k + k * ld];
              for (int q = 0; q < k; ++q) sv[q] -= sv[k] * H[q + k * ld];
            }
        }
      }
      __syncthreads();
      if (g.status != 0) break;
      {
        const int gi = g.gi;
        ens_rows<CTAS>(n, gtid, [&](int, int q) {
          double xe = x[q];
          for (int j = 0; j < gi; ++j) {
            const double sj = sv[j];
            if (sj != 0) xe += sj * Z[(size_t)j * n + q];
          }
          x[q] = xe;
        });
      }
      cluster.sync();  // x complete before the residual gathers it
      if (lead) g.iter++;
      __syncthreads();
    }
    if (!walked) {
      if (gtid == 0) {
        atomicExch(e.abort, 1);
        e.res[mi] = EnsResult{g.resid, g.initR, g.iter, RSG_TIMEOUT, inner};
      }
      return;
    }
    cluster.sync();  // every CTA is done with this member's vectors and g
    if (gtid == 0)
      e.res[mi] = EnsResult{g.resid, g.initR, g.iter, g.status == KS_CONVERGED ? RSG_OK : -g.status, inner};
    __syncthreads();
  }
}

// One solver state per device: its own stream, descriptor table and
// workspace, grown as ensembles need.
struct EnsDevice {
  std::mutex mu;
  cudaStream_t stream = nullptr;
  DeviceBuffer<EnsMember> mem;
  DeviceBuffer<EnsResult> res;
  DeviceBuffer<int> ctl;
  DeviceBuffer<int> errs;  // per instance: a walk's timeout flag (written only by its own cluster)
  DeviceBuffer<double> work;
  DeviceBuffer<float> workf;
  std::map<int, int> max_clusters;  // per kernel variant: clusters resident at once (0: not schedulable)
};

std::mutex g_ens_mu;
std::map<int, std::unique_ptr<EnsDevice>> g_ens;

using EnsKernel = void (*)(EnsArgs, size_t);

int ens_clusters(EnsDevice& D, int key, EnsKernel kern, int ctas) {
  auto it = D.max_clusters.find(key);
  if (it != D.max_clusters.end()) return it->second;
  int nclusters = 0;
  bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RING_SMEM_MAX) ==
            cudaSuccess;
  if (ok && ctas > 8)
    ok = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(ENS_THREADS);
    cfg.dynamicSmemBytes = RING_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaOccupancyMaxActiveClusters(&nclusters, (const void*)kern, &cfg) != cudaSuccess) nclusters = 0;
  }
  cudaGetLastError();
  D.max_clusters[key] = nclusters;
  return nclusters;
}

void ens_launch(EnsDevice& D, int count, int key, EnsKernel kern, int ctas, size_t smem, size_t ring_bytes) {
  const int fit = ens_clusters(D, key, kern, ctas);
  if (fit < 1) throw Error(RSG_UNSUPPORTED, "the ensemble solver's clusters cannot be scheduled on this device");
  if (smem > RING_SMEM_MAX) throw Error(RSG_UNSUPPORTED, "walk schedule too deep for the ensemble solver");
  const int nclusters = std::min(count, fit);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas * nclusters);
  cfg.blockDim = dim3(ENS_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = D.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  EnsArgs a{count, D.mem.get(), D.res.get(), D.ctl.get(), D.ctl.get() + 1};
  RSG_CUDA(cudaLaunchKernelEx(&cfg, kern, a, ring_bytes));
}

}  // namespace

void ensemble_solve(const std::vector<EnsSystem>& sys, int precision, std::vector<rsg_solve_info>& info,
                    std::vector<int>& status) {
  const int count = (int)sys.size();
  info.assign(count, rsg_solve_info{});
  status.assign(count, RSG_OK);
  if (count == 0) return;
  if (precision != 0 && precision != 1) throw Error(RSG_BAD_ARG, "precision must be 0 (FP64) or 1 (mixed)");
  const int device = sys[0].ctx->device;
  // members the kernel cannot take are reported one by one; the rest run
  std::vector<int> idx;
  std::vector<EnsMember> h;
  int C = 0, R = 0, mr = 0;
  size_t nw = 0, nf = 0;
  // 8-CTA clusters when planned and there are more members than 16-CTA
  // clusters run at once: twice as many members in flight (measured on 152
  // SMs: with 16-CTA clusters one to four members took the same time and
  // eight took twice as long; with 8-CTA clusters one to nine took the same
  // time).  A few members alone are faster on 16 SMs each (a 96x96x24 member:
  // 3.6 against 4.7 ms per iteration).
  const int prefer = count > 4 ? 8 : 16;
  for (int i = 0; i < count; ++i) {
    const EnsSystem& q = sys[i];
    SolverView sv = solver_view(*q.solver);
    const RingPlan *L = nullptr, *U = nullptr;
    if (q.ctx->device != device) {
      status[i] = RSG_BAD_ARG;  // members must share one device
      continue;
    }
    if (sv.setup_for != q.A) {
      status[i] = RSG_BAD_ARG;  // the solver must have been set up with this matrix
      continue;
    }
    if (sv.method != RSG_BICGSTAB || sv.pc_kind != RSG_PC_ILU || !ilu_ring_plans(sv.pc, prefer, &L, &U) ||
        (C != 0 && (L->C != C || U->C != C)) || (L->C != 8 && L->C != 16) || U->C != L->C) {
      status[i] = RSG_UNSUPPORTED;  // BiCGstab + ILU(0) with level-walk schedules for one cluster shape
      continue;
    }
    C = L->C;
    R = std::max({R, L->R, U->R});
    Csr& A = *q.A;
    A.refresh_sell();
    EnsMember m{};
    m.n = A.n;
    m.sb = A.slice_base.get();
    m.rl = A.row_len.get();
    m.col = A.sell_col.get();
    m.val = A.sell_val.get();
    m.gl = RingArgs{L->nlev,    L->R,        L->slack,        L->slice_base.get(), L->row.get(), L->len.get(),
                    L->ridx.get(), L->pmask.get(), L->expect.get(), L->nbr.get(),       nullptr};
    m.gu = RingArgs{U->nlev,    U->R,        U->slack,        U->slice_base.get(), U->row.get(), U->len.get(),
                    U->ridx.get(), U->pmask.get(), U->expect.get(), U->nbr.get(),       nullptr};
    m.lval = L->val.get();
    m.uval = U->val.get();
    m.udiag = U->diag.get();
    m.lvalf = L->valf.get();
    m.uvalf = U->valf.get();
    m.udiagf = U->diagf.get();
    m.b = q.b;
    m.x = q.x;
    m.rtol = sv.rtol;
    m.atol = sv.atol;
    m.dtol = sv.dtol;
    m.maxIter = sv.maxIter;
    m.restart = std::max(1, sv.restart);
    m.inner_iters = sv.inner_iters;
    m.inner_rtol = sv.inner_rtol;
    if (precision) {
      A.refresh_sell_f32();
      m.valf = A.sell_valf.get();
      mr = std::max(mr, m.restart);
    }
    nw += (size_t)A.n * (precision ? (size_t)(3 + 2 * m.restart) : 9);
    nf += precision ? (size_t)A.n * 10 : 0;
    RSG_CUDA(cudaStreamSynchronize(q.ctx->stream));  // matrix, factors and b are ready
    idx.push_back(i);
    h.push_back(m);
  }
  const int nrun = (int)idx.size();
  if (nrun == 0) return;
  // largest systems first: the clusters take members in this order, so the
  // launch does not end waiting for a big member taken last
  {
    std::vector<int> ord(nrun);
    for (int k = 0; k < nrun; ++k) ord[k] = k;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return h[a].n > h[b].n; });
    std::vector<int> idx2(nrun);
    std::vector<EnsMember> h2(nrun);
    for (int k = 0; k < nrun; ++k) {
      idx2[k] = idx[ord[k]];
      h2[k] = h[ord[k]];
    }
    idx.swap(idx2);
    h.swap(h2);
  }
  // shared memory: the ring of the walks (FP64 or FP32 values), then for
  // FGMRES the Hessenberg matrix, right-hand side and rotations
  const size_t ring_bytes = precision ? ring_smem_bytes<float>(R) : ring_smem_bytes<double>(R);
  const size_t smem = ring_bytes + (precision ? sizeof(double) * ((size_t)(mr + 1) * mr + 3 * (size_t)(mr + 1)) : 0);
  EnsDevice* D;
  {
    std::lock_guard<std::mutex> lk(g_ens_mu);
    auto& slot = g_ens[device];
    if (!slot) slot.reset(new EnsDevice);
    D = slot.get();
  }
  std::lock_guard<std::mutex> lk(D->mu);
  RSG_CUDA(cudaSetDevice(device));
  if (!D->stream) RSG_CUDA(cudaStreamCreateWithFlags(&D->stream, cudaStreamNonBlocking));
  if (D->work.size() < nw) D->work.resize(nw);
  if (nf && D->workf.size() < nf) D->workf.resize(nf);
  size_t off = 0, offf = 0;
  for (int i = 0; i < nrun; ++i) {
    h[i].w = D->work.get() + off;
    h[i].f = precision ? D->workf.get() + offf : nullptr;
    off += (size_t)h[i].n * (precision ? (size_t)(3 + 2 * h[i].restart) : 9);
    offf += precision ? (size_t)h[i].n * 10 : 0;
  }
  if (D->mem.size() < (size_t)nrun) D->mem.resize(nrun);
  if (D->res.size() < (size_t)nrun) D->res.resize(nrun);
  if (D->ctl.size() < 2) D->ctl.resize(2);
  if (D->errs.size() < (size_t)nrun) D->errs.resize(nrun);
  for (int k = 0; k < nrun; ++k) h[k].gl.err = h[k].gu.err = D->errs.get() + k;
  RSG_CUDA(cudaMemsetAsync(D->errs.get(), 0, sizeof(int) * nrun, D->stream));
  RSG_CUDA(cudaMemcpyAsync(D->mem.get(), h.data(), sizeof(EnsMember) * nrun, cudaMemcpyHostToDevice, D->stream));
  // instances no cluster reaches (after a walk timed out) report the timeout
  std::vector<EnsResult> hr(nrun, EnsResult{0, 0, 0, RSG_TIMEOUT, 0});
  RSG_CUDA(cudaMemcpyAsync(D->res.get(), hr.data(), sizeof(EnsResult) * nrun, cudaMemcpyHostToDevice, D->stream));
  RSG_CUDA(cudaMemsetAsync(D->ctl.get(), 0, 2 * sizeof(int), D->stream));
  const int key = precision * 100 + C;
  EnsKernel kern = nullptr;
  if (C == 16) kern = precision ? k_ens_fgmres<16> : k_ens_bicgstab<16>;
  else if (C == 8) kern = precision ? k_ens_fgmres<8> : k_ens_bicgstab<8>;
  else throw Error(RSG_UNSUPPORTED, "ensemble walk schedules must be for clusters of 8 or 16 CTAs");
  ens_launch(*D, nrun, key, kern, C, smem, ring_bytes);
  RSG_CUDA(cudaMemcpyAsync(hr.data(), D->res.get(), sizeof(EnsResult) * nrun, cudaMemcpyDeviceToHost, D->stream));
  RSG_CUDA(cudaStreamSynchronize(D->stream));
  RSG_CUDA(cudaGetLastError());
  for (int k = 0; k < nrun; ++k) {
    const int i = idx[k];
    info[i].iterations = hr[k].iterations;
    info[i].residual = hr[k].residual;
    info[i].initial_residual = hr[k].initR;
    info[i].inner_iterations = hr[k].inner;
    info[i].reason = hr[k].status;
    status[i] = hr[k].status;
  }
}

}  // namespace rsg

using rsg::guarded;

extern "C" {

rsg_status rsg_solver_solve_batched(int32_t count, rsg_solver* const* solvers, rsg_csr* const* A,
                                    const double* const* b, double* const* x, int32_t precision,
                                    rsg_solve_info* infos, int32_t* statuses) {
  if (count < 0 || (count > 0 && (!solvers || !A || !b || !x))) return RSG_BAD_ARG;
  if (precision != 0 && precision != 1) return RSG_BAD_ARG;
  for (int i = 0; i < count; ++i)
    if (!solvers[i] || !A[i] || !b[i] || !x[i]) return RSG_BAD_ARG;
  if (count == 0) return RSG_OK;
  std::vector<rsg::DeviceBuffer<double>> db(count), dx(count);
  std::vector<rsg::EnsSystem> sys(count);
  rsg::Context* ctx0 = nullptr;
  std::vector<rsg_status> st(count, RSG_OK);
  for (int i = 0; i < count; ++i) {
    rsg::Context* ctx = rsg::solver_view(*solvers[i]->s).ctx;
    if (!ctx0) ctx0 = ctx;
    const int n = A[i]->m.n;
    st[i] = guarded(ctx, [&] {
      db[i].resize(n);
      dx[i].resize(n);
      RSG_CUDA(cudaMemcpyAsync(db[i].get(), b[i], sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
      RSG_CUDA(cudaMemcpyAsync(dx[i].get(), x[i], sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    });
    sys[i] = rsg::EnsSystem{ctx, &A[i]->m, solvers[i]->s.get(), db[i].get(), dx[i].get()};
  }
  std::vector<rsg_solve_info> si;
  std::vector<int> ss;
  rsg_status e = guarded(ctx0, [&] { rsg::ensemble_solve(sys, precision, si, ss); });
  rsg_status first = RSG_OK;
  for (int i = 0; i < count; ++i) {
    rsg::Context* ctx = sys[i].ctx;
    rsg_status r = st[i] != RSG_OK ? st[i] : (e != RSG_OK ? e : (rsg_status)ss[i]);
    // as rsg_solver_solve: x as it stood at the end, copied back either way
    rsg_status c = guarded(ctx, [&] {
      RSG_CUDA(cudaMemcpyAsync(x[i], dx[i].get(), sizeof(double) * A[i]->m.n, cudaMemcpyDeviceToHost, ctx->stream));
      ctx->sync();
    });
    if (r == RSG_OK) r = c;
    if (infos) {
      infos[i] = e == RSG_OK ? si[i] : rsg_solve_info{};
      infos[i].reason = r;
    }
    if (statuses) statuses[i] = r;
    if (first == RSG_OK) first = r;
  }
  return first;
}

}  // extern "C"

