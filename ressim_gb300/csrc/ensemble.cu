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
// Inside a cluster:
// * SpMV, BLAS-1 and the BiCGstab recurrences run over the cluster's 2,048
//   threads (thread t owns rows t, t + 2048, ...); values that other SMs
//   wrote earlier in the launch (the walks' outputs, the vectors the walks
//   read) are loaded from L2 (ld.global.cg), never from a possibly stale L1
//   line or the read-only cache;
// * dot products reduce per warp, then across the cluster's 64 warps
//   through distributed shared memory in a fixed tree, so every CTA holds
//   the same scalars and the result does not depend on the cluster shape
//   (16 CTAs of 4 warps or 8 CTAs of 8 warps give identical bits);
// * the ILU(0) triangular solves are the level walks of ring.cuh, in FP64
//   (plain mode) or on the FP32 copies of the factors (mixed precision: the
//   Krylov vectors, SpMV, dots and updates stay FP64; BiCGstab's recursively
//   updated residual equals b - A x whatever the preconditioner applies, so
//   the FP64 stopping test keeps its meaning).
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
  double* w;  // 9 vectors of n: r, rtilde, p, v, phat, s, shat, t, y
  float* f;   // 3 vectors of n (FP32 walks)
  double rtol, atol, dtol;
  int maxIter;
};

struct EnsResult {
  double residual, initR;
  int iterations, status;
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

// Sum of K per-thread values over the cluster; every thread gets the total.
// part: shared [2][3][warps per CTA], tot: shared [3]; ph alternates the two
// halves of part so one barrier per reduction suffices.
template <int CTAS, int K>
__device__ __forceinline__ void cluster_sum(double (&v)[K], double* part, double* tot, int& ph,
                                            cg::cluster_group& cluster) {
  constexpr int WPC = RING_SLICES / CTAS;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) part[(ph * 3 + q) * WPC + w] = x;
  }
  cluster.sync();
  if (w == 0) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      // the 64 warps of the cluster in global order: lane l adds warps l and l + 32
      const int g0 = lane, g1 = lane + 32;
      const double* p0 = cluster.map_shared_rank(part + (ph * 3 + q) * WPC + g0 % WPC, g0 / WPC);
      const double* p1 = cluster.map_shared_rank(part + (ph * 3 + q) * WPC + g1 % WPC, g1 / WPC);
      double x = *p0 + *p1;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) tot[q] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < K; ++q) v[q] = tot[q];
  ph ^= 1;
}

// A walk as a called function: its registers are allocated apart from the
// solver loop's, which keeps both free of spills.
// (13 entries of a row in registers, as for the 27-point stencil; longer
// rows read the rest from memory)
template <int KIND, typename T, int CTAS>
__device__ __noinline__ bool walk(const RingArgs& g, const RingVals<T>& a, unsigned char* smem) {
  return ring_walk<KIND, T, 13, CTAS>(g, a, smem);
}

// out = M^-1 in (ILU(0): L y = in, U out = y) on the cluster; ends with a
// cluster barrier, so out is complete for every thread of the cluster.
template <typename TW, int CTAS>
__device__ __noinline__ bool ens_precond(const EnsMember& m, const double* in, double* out, unsigned char* smem,
                                            int gtid, int nt, cg::cluster_group& cluster) {
  const int n = m.n;
  if constexpr (sizeof(TW) == 4) {
    float *fb = m.f, *fy = m.f + n, *fz = m.f + 2 * (size_t)n;
    for (int i = gtid; i < n; i += nt) fb[i] = (float)in[i];
    // the walk starts with a cluster barrier, which publishes fb
    const RingVals<float> lo{m.lvalf, nullptr, fb, fy, nullptr};
    if (!walk<SW_ILU_LOWER, float, CTAS>(m.gl, lo, smem)) return false;
    const RingVals<float> up{m.uvalf, m.udiagf, fy, fz, nullptr};
    if (!walk<SW_ILU_UPPER, float, CTAS>(m.gu, up, smem)) return false;
    for (int i = gtid; i < n; i += nt) out[i] = (double)__ldcg(fz + i);
  } else {
    double* y = m.w + 8 * (size_t)n;
    const RingVals<double> lo{m.lval, nullptr, in, y, nullptr};
    if (!walk<SW_ILU_LOWER, double, CTAS>(m.gl, lo, smem)) return false;
    const RingVals<double> up{m.uval, m.udiag, y, out, nullptr};
    if (!walk<SW_ILU_UPPER, double, CTAS>(m.gu, up, smem)) return false;
  }
  cluster.sync();
  return true;
}

template <typename TW, int CTAS>
__global__ void __launch_bounds__(RING_SLICES / CTAS * 32) k_ens_bicgstab(EnsArgs e) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double part[2 * 3 * (RING_SLICES / CTAS)];
  __shared__ double tot[3];
  __shared__ int take;
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int nt = CTAS * (int)blockDim.x, gtid = rank * (int)blockDim.x + (int)threadIdx.x;
  int ph = 0;
  for (;;) {
    if (rank == 0 && threadIdx.x == 0) take = *(volatile int*)e.abort ? e.count : atomicAdd(e.queue, 1);
    cluster.sync();
    const int mi = *cluster.map_shared_rank(&take, 0);
    cluster.sync();  // CTA 0 rewrites take only after every CTA has read it
    if (mi >= e.count) return;
    const EnsMember& m = e.mem[mi];
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
      double a2[2] = {0, 0};
      for (int i = gtid; i < n; i += nt) {
        const int base = m.sb[i >> 5] + (i & 31), len = m.rl[i];
        double d = 0;
        for (int k = 0; k < len; ++k) {
          const int q = base + 32 * k;
          d += m.val[q] * __ldcg(x + m.col[q]);
        }
        const double ri = m.b[i] + -1.0 * d;
        r[i] = ri;
        rt[i] = ri;
        a2[0] += ri * ri;
        a2[1] += ri * ri;
      }
      cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
      top(a2[0], a2[1]);
    }
    while (status == KS_RUNNING) {
      // p = r + beta (p - omega v)
      for (int i = gtid; i < n; i += nt) {
        if (first) {
          p[i] = r[i];
          continue;
        }
        const double mo = -omega;
        double temp = (mo == 0) ? 0.0 : mo * v[i];
        temp += p[i];
        p[i] = (beta == 0) ? r[i] : r[i] + beta * temp;
      }
      if (!(walked = ens_precond<TW, CTAS>(m, p, phat, smem, gtid, nt, cluster))) break;
      {
        // v = A phat; alpha = rho_1 / (rtilde . v)
        double a1[1] = {0};
        for (int i = gtid; i < n; i += nt) {
          const double d = sell_row_fma<false>(m.val, m.col, phat, m.sb[i >> 5] + (i & 31), m.rl[i]);
          const double yi = (d != 0) ? d : 0.0;
          v[i] = yi;
          a1[0] = __fma_rn(rt[i], yi, a1[0]);
        }
        cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
        alpha = rho_1 / a1[0];
      }
      {
        // s = r - alpha v; monitor |s|
        double a1[1] = {0};
        const double ma = -alpha;
        for (int i = gtid; i < n; i += nt) {
          const double si = (ma == 0) ? r[i] : r[i] + ma * v[i];
          s[i] = si;
          a1[0] += si * si;
        }
        cluster_sum<CTAS, 1>(a1, part, tot, ph, cluster);
        const int mo = monitor(sqrt(a1[0]));
        if (mo == 1) {
          // x.add(alpha, phat) and stop
          if (alpha != 0)
            for (int i = gtid; i < n; i += nt) x[i] += alpha * __ldcg(phat + i);
          status = KS_CONVERGED;
          break;
        }
        if (mo < 0) {
          status = mo;
          break;
        }
      }
      if (!(walked = ens_precond<TW, CTAS>(m, s, shat, smem, gtid, nt, cluster))) break;
      {
        // t = A shat; omega = (t . s) / (t . t)
        double a2[2] = {0, 0};
        for (int i = gtid; i < n; i += nt) {
          const double d = sell_row_fma<false>(m.val, m.col, shat, m.sb[i >> 5] + (i & 31), m.rl[i]);
          const double yi = (d != 0) ? d : 0.0;
          t[i] = yi;
          a2[0] = __fma_rn(yi, s[i], a2[0]);
          a2[1] = __fma_rn(yi, yi, a2[1]);
        }
        cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
        omega = a2[0] / a2[1];
      }
      {
        // x += alpha phat + omega shat; r = s - omega t; reduce r.r, rtilde.r
        double a2[2] = {0, 0};
        const double mo = -omega;
        for (int i = gtid; i < n; i += nt) {
          double xi = x[i];
          if (alpha != 0) xi += alpha * __ldcg(phat + i);
          if (omega != 0) xi += omega * __ldcg(shat + i);
          x[i] = xi;
          const double ri = (mo == 0) ? s[i] : s[i] + mo * t[i];
          r[i] = ri;
          a2[0] += ri * ri;
          a2[1] += rt[i] * ri;
        }
        cluster_sum<CTAS, 2>(a2, part, tot, ph, cluster);
        rho_2 = rho_1;
        iter++;
        first = 0;
        top(a2[0], a2[1]);
      }
    }
    if (!walked) {
      if (gtid == 0) {
        atomicExch(e.abort, 1);
        e.res[mi] = EnsResult{resid, initR, iter, RSG_TIMEOUT};
      }
      return;  // this cluster's shared memory may still receive pushes
    }
    cluster.sync();  // the last updates of x are in place before the next instance
    if (gtid == 0) e.res[mi] = EnsResult{resid, initR, iter, status == KS_CONVERGED ? RSG_OK : -status};
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

template <typename TW, int CTAS>
int ens_clusters(EnsDevice& D, int key) {
  auto it = D.max_clusters.find(key);
  if (it != D.max_clusters.end()) return it->second;
  auto kern = k_ens_bicgstab<TW, CTAS>;
  int nclusters = 0;
  bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RING_SMEM_MAX) ==
            cudaSuccess;
  if (ok && CTAS > 8)
    ok = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CTAS);
    cfg.blockDim = dim3(RING_SLICES / CTAS * 32);
    cfg.dynamicSmemBytes = RING_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CTAS;
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

template <typename TW, int CTAS>
void ens_launch(EnsDevice& D, int count, int key, size_t smem) {
  const int fit = ens_clusters<TW, CTAS>(D, key);
  if (fit < 1) throw Error(RSG_UNSUPPORTED, "the ensemble solver's clusters cannot be scheduled on this device");
  const int nclusters = std::min(count, fit);
  auto kern = k_ens_bicgstab<TW, CTAS>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CTAS * nclusters);
  cfg.blockDim = dim3(RING_SLICES / CTAS * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = D.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CTAS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  EnsArgs a{count, D.mem.get(), D.res.get(), D.ctl.get(), D.ctl.get() + 1};
  RSG_CUDA(cudaLaunchKernelEx(&cfg, kern, a));
}

}  // namespace

void ensemble_solve(const std::vector<EnsSystem>& sys, int precision, std::vector<rsg_solve_info>& info,
                    std::vector<int>& status) {
  const int count = (int)sys.size();
  info.assign(count, rsg_solve_info{});
  status.assign(count, RSG_OK);
  if (count == 0) return;
  if (precision != 0 && precision != 1) throw Error(RSG_BAD_ARG, "precision must be 0 (FP64) or 1 (FP32 factors)");
  const int device = sys[0].ctx->device;
  // members the kernel cannot take are reported one by one; the rest run
  std::vector<int> idx;
  std::vector<EnsMember> h;
  int C = 0, R = 0;
  size_t nw = 0;
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
    if (sv.method != RSG_BICGSTAB || sv.pc_kind != RSG_PC_ILU || !ilu_ring_plans(sv.pc, &L, &U) ||
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
    nw += (size_t)A.n;
    RSG_CUDA(cudaStreamSynchronize(q.ctx->stream));  // matrix, factors and b are ready
    idx.push_back(i);
    h.push_back(m);
  }
  const int nrun = (int)idx.size();
  if (nrun == 0) return;
  const size_t smem = precision ? ring_smem_bytes<float>(R) : ring_smem_bytes<double>(R);
  if (smem > RING_SMEM_MAX) throw Error(RSG_UNSUPPORTED, "walk schedule too deep for the ensemble solver");
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
  if (D->work.size() < nw * 9) D->work.resize(nw * 9);
  if (precision && D->workf.size() < nw * 3) D->workf.resize(nw * 3);
  size_t off = 0;
  for (int i = 0; i < nrun; ++i) {
    h[i].w = D->work.get() + off * 9;
    h[i].f = precision ? D->workf.get() + off * 3 : nullptr;
    off += (size_t)h[i].n;
  }
  if (D->mem.size() < (size_t)nrun) D->mem.resize(nrun);
  if (D->res.size() < (size_t)nrun) D->res.resize(nrun);
  if (D->ctl.size() < 2) D->ctl.resize(2);
  if (D->errs.size() < (size_t)nrun) D->errs.resize(nrun);
  for (int k = 0; k < nrun; ++k) h[k].gl.err = h[k].gu.err = D->errs.get() + k;
  RSG_CUDA(cudaMemsetAsync(D->errs.get(), 0, sizeof(int) * nrun, D->stream));
  RSG_CUDA(cudaMemcpyAsync(D->mem.get(), h.data(), sizeof(EnsMember) * nrun, cudaMemcpyHostToDevice, D->stream));
  // instances no cluster reaches (after a walk timed out) report the timeout
  std::vector<EnsResult> hr(nrun, EnsResult{0, 0, 0, RSG_TIMEOUT});
  RSG_CUDA(cudaMemcpyAsync(D->res.get(), hr.data(), sizeof(EnsResult) * nrun, cudaMemcpyHostToDevice, D->stream));
  RSG_CUDA(cudaMemsetAsync(D->ctl.get(), 0, 2 * sizeof(int), D->stream));
  const int key = precision * 100 + C;
  if (C == 16) {
    if (precision) ens_launch<float, 16>(*D, nrun, key, smem);
    else ens_launch<double, 16>(*D, nrun, key, smem);
  } else if (C == 8) {
    if (precision) ens_launch<float, 8>(*D, nrun, key, smem);
    else ens_launch<double, 8>(*D, nrun, key, smem);
  } else
    throw Error(RSG_UNSUPPORTED, "ensemble walk schedules must be for clusters of 8 or 16 CTAs");
  RSG_CUDA(cudaMemcpyAsync(hr.data(), D->res.get(), sizeof(EnsResult) * nrun, cudaMemcpyDeviceToHost, D->stream));
  RSG_CUDA(cudaStreamSynchronize(D->stream));
  RSG_CUDA(cudaGetLastError());
  for (int k = 0; k < nrun; ++k) {
    const int i = idx[k];
    info[i].iterations = hr[k].iterations;
    info[i].residual = hr[k].residual;
    info[i].initial_residual = hr[k].initR;
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

