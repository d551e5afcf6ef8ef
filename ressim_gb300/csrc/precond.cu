// Preconditioners: ILU(0) (mtj/src/no/uib/cipr/matrix/sparse/ILU.java:54-140
// with UnitLowerCompRowMatrix.java:48-86 and UpperCompRowMatrix.java:48-90),
// SSOR (sparse/SSOR.java:126-194) and the diagonal preconditioner
// (sparse/DiagonalPreconditioner.java:44-78).
//
// The sequential sweeps are level scheduled: rows are grouped by the depth
// of their dependency chain, every row is computed by one thread that sums
// its entries in CSR order (so each row's arithmetic equals the Java loop),
// and one thread-block cluster walks the levels with a hardware cluster
// barrier between them.  Coefficients are stored per level as SELL-32 slices
// so the loads of a warp are contiguous.
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <cstdlib>
#include <string>

#include "ring.cuh"

namespace rsg {

template <typename T>
struct SweepArgs {
  int nlev;
  const int* level_slices;
  const int* slice_base;
  const int* row;
  const int* len;
  const int* col;
  const T* val;
  const T* diag;
  const T* b;
  T* x;   // output / in-place vector
  T* xx;  // SSOR half iterate
  T omega;
  const int* active;
};

__device__ __forceinline__ double ld_l2(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float ld_l2(const float* p) { return __ldcg(p); }
__device__ __forceinline__ void st_l2(double* p, double v) { __stcg(p, v); }
__device__ __forceinline__ void st_l2(float* p, float v) { __stcg(p, v); }

template <int KIND, typename T>
__device__ __forceinline__ void sweep_row(const SweepArgs<T>& a, int slot, int row, int s) {
  const int base = a.slice_base[s] + (slot & 31);
  const int len = a.len[slot];
  T sum = 0;
  if constexpr (KIND == SW_SSOR_FWD || KIND == SW_SSOR_BWD) {
    // sigma over the full row without the diagonal, CSR order; lower
    // columns read the half iterate xx, upper columns read x.
#pragma unroll 4
    for (int k = 0; k < len; ++k) {
      int q = base + 32 * k;
      int c = a.col[q];
      T v = (c < row) ? ld_l2(a.xx + c) : ld_l2(a.x + c);
      sum += a.val[q] * v;
    }
    T d = a.diag[slot];
    T sigma = (a.b[row] - sum) / d;
    if (KIND == SW_SSOR_FWD) {
      T xo = ld_l2(a.x + row);
      st_l2(a.xx + row, xo + a.omega * (sigma - xo));
    } else {
      T xh = ld_l2(a.xx + row);
      st_l2(a.x + row, xh + a.omega * (sigma - xh));
    }
  } else {
#pragma unroll 4
    for (int k = 0; k < len; ++k) {
      int q = base + 32 * k;
      sum += a.val[q] * ld_l2(a.x + a.col[q]);
    }
    if (KIND == SW_ILU_LOWER) st_l2(a.x + row, a.b[row] - sum);
    else st_l2(a.x + row, (a.b[row] - sum) / a.diag[slot]);
  }
}

// One cluster walks all levels.  Every CTA of the cluster evaluates the same
// early-exit test, so either all of them reach each barrier or none does.
template <int KIND, typename T>
__global__ void __launch_bounds__(512) k_sweep_cluster(SweepArgs<T> a) {
  if (a.active && *a.active != 0) return;
  cg::cluster_group cluster = cg::this_cluster();
  const int wpc = blockDim.x >> 5;
  const int gwarp = (int)cluster.block_rank() * wpc + (threadIdx.x >> 5);
  const int nwarps = (int)cluster.num_blocks() * wpc;
  const int lane = threadIdx.x & 31;
  for (int l = 0; l < a.nlev; ++l) {
    const int s1 = a.level_slices[l + 1];
    for (int s = a.level_slices[l] + gwarp; s < s1; s += nwarps) {
      const int slot = s * 32 + lane;
      const int row = a.row[slot];
      if (row >= 0) sweep_row<KIND, T>(a, slot, row, s);
    }
    cluster.sync();
  }
}

// ILU sweeps with a three-stage software pipeline per warp: slot metadata
// (row id, length, slice base) is loaded two levels ahead, the coefficients,
// column indices, right-hand side and diagonal one level ahead, and only the
// gathers of already-computed x values (L2 hits written by the previous
// levels) remain between two cluster barriers.  Loads are predicated rather
// than branched on, so issuing them never waits for earlier loads.  Rows are
// summed in CSR order as in the sequential loop.  Each warp owns one slice
// per level; levels with more slices than warps take the remaining slices
// through the plain path.
struct SlotMeta {
  int row, len, base;
};

template <typename T, int MAXW>
struct RowPrefetch {
  int row, len, base;
  T b, d;
  T v[MAXW];
  int c[MAXW];
};

template <typename T>
__device__ __forceinline__ SlotMeta load_meta(const SweepArgs<T>& a, const int* ls, int l, int gwarp, int lane) {
  SlotMeta m{-1, 0, 0};
  if (l >= a.nlev) return m;
  const int s = ls[l] + gwarp;
  if (s >= ls[l + 1]) return m;
  const int slot = s * 32 + lane;
  m.row = a.row[slot];
  m.len = a.len[slot];
  m.base = a.slice_base[s] + lane;
  return m;
}

template <int KIND, typename T, int MAXW>
__device__ __forceinline__ void load_coeffs(const SweepArgs<T>& a, const int* ls, const SlotMeta& m, int l, int gwarp,
                                            int lane, RowPrefetch<T, MAXW>& p) {
  p.row = m.row;
  p.len = m.row >= 0 ? m.len : 0;
  p.base = m.base;
  const int r = m.row >= 0 ? m.row : 0;
  p.b = a.b[r];
  if (KIND == SW_ILU_UPPER) {
    const int s = (m.row >= 0) ? ls[l] + gwarp : 0;
    p.d = a.diag[s * 32 + lane];
  }
#pragma unroll
  for (int k = 0; k < MAXW; ++k)
    if (k < p.len) {
      p.v[k] = a.val[p.base + 32 * k];
      p.c[k] = a.col[p.base + 32 * k];
    }
}

template <int KIND, typename T, int MAXW>
__device__ __forceinline__ void finish_row(const SweepArgs<T>& a, const RowPrefetch<T, MAXW>& p) {
  if (p.row < 0) return;
  T xv[MAXW];
#pragma unroll
  for (int k = 0; k < MAXW; ++k)
    if (k < p.len) xv[k] = ld_l2(a.x + p.c[k]);
  T sum = 0;
#pragma unroll
  for (int k = 0; k < MAXW; ++k)
    if (k < p.len) sum += p.v[k] * xv[k];
  for (int k = MAXW; k < p.len; ++k) {
    int q = p.base + 32 * k;
    sum += a.val[q] * ld_l2(a.x + a.col[q]);
  }
  if (KIND == SW_ILU_LOWER) st_l2(a.x + p.row, p.b - sum);
  else st_l2(a.x + p.row, (p.b - sum) / p.d);
}

constexpr int SWEEP_MAX_LEVELS = 8192;  // level offsets staged in shared memory

template <int KIND, typename T, int MAXW>
__global__ void __launch_bounds__(256) k_sweep_pipelined(SweepArgs<T> a) {
  if (a.active && *a.active != 0) return;
  __shared__ int ls[SWEEP_MAX_LEVELS + 1];
  for (int q = threadIdx.x; q <= a.nlev; q += blockDim.x) ls[q] = a.level_slices[q];
  __syncthreads();
  cg::cluster_group cluster = cg::this_cluster();
  const int wpc = blockDim.x >> 5;
  const int gwarp = (int)cluster.block_rank() * wpc + (threadIdx.x >> 5);
  const int nwarps = (int)cluster.num_blocks() * wpc;
  const int lane = threadIdx.x & 31;
  RowPrefetch<T, MAXW> cur, nxt;
  SlotMeta m1 = load_meta(a, ls, 1, gwarp, lane);
  {
    SlotMeta m0 = load_meta(a, ls, 0, gwarp, lane);
    load_coeffs<KIND, T, MAXW>(a, ls, m0, 0, gwarp, lane, cur);
  }
  for (int l = 0; l < a.nlev; ++l) {
    const SlotMeta m2 = load_meta(a, ls, l + 2, gwarp, lane);
    load_coeffs<KIND, T, MAXW>(a, ls, m1, l + 1, gwarp, lane, nxt);
    finish_row<KIND, T, MAXW>(a, cur);
    const int s1 = ls[l + 1];
    for (int s = ls[l] + gwarp + nwarps; s < s1; s += nwarps) {
      const int slot = s * 32 + lane;
      const int row = a.row[slot];
      if (row >= 0) sweep_row<KIND, T>(a, slot, row, s);
    }
    cluster.sync();
    cur = nxt;
    m1 = m2;
  }
}

// RSG_SWEEP=pipelined switches the ring walks off; RSG_RING_CTAS=8 or 16
// plans them for that cluster shape only (8 CTAs of 8 warps, 16 of 4);
// otherwise both are planned and the walk autotuner picks.
static bool ring_enabled() {
  static const bool on = [] {
    const char* e = getenv("RSG_SWEEP");
    return !(e && std::string(e) == "pipelined");
  }();
  return on;
}

static int ring_ctas() {
  static const int c = [] {
    const char* e = getenv("RSG_RING_CTAS");
    return e ? (atoi(e) == 8 ? 8 : (atoi(e) == 16 ? 16 : 0)) : 0;
  }();
  return c;
}

// Fallback: one launch per level.
template <int KIND, typename T>
__global__ void k_sweep_level(SweepArgs<T> a, int l) {
  if (a.active && *a.active != 0) return;
  const int s = a.level_slices[l] + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s >= a.level_slices[l + 1]) return;
  const int slot = s * 32 + (threadIdx.x & 31);
  const int row = a.row[slot];
  if (row >= 0) sweep_row<KIND, T>(a, slot, row, s);
}

// ILU(0) factorisation, one thread per row, rows of a level in parallel.
// Row k reads only rows of earlier levels (its lower neighbours), which are
// final once the barrier of their level has passed.
// The elimination of row k is a fixed program of the pattern: for every
// lower entry i (ascending) the pairs (l, j) with data[l] -= LUki * data[j]
// in the order of the merge scan of ILU.java:113-120.  The host lists those
// pairs once per pattern (upd_ptr indexed by CSR position, upd_l, upd_j), so
// the device only streams them.
struct FactorArgs {
  int nlev;
  const int* level_slices;
  const int* row;
  const int* rowptr;
  const int* col;
  const int* diag;
  const int* upd_ptr;
  const int* upd_l;
  const int* upd_j;
  double* data;
  int* flag;  // first zero-pivot row + 1
};

constexpr int FACTOR_ROW_MAX = 32;  // rows up to this length keep their values in a local array
constexpr int FACTOR_BATCH = 16;

__device__ __forceinline__ void factor_row_global(const FactorArgs& a, int k) {
  const int r0 = a.rowptr[k], dk = a.diag[k];
  for (int i = r0; i < dk; ++i) {
    const int index = a.col[i];
    const double LUii = ld_l2(a.data + a.diag[index]);
    if (LUii == 0) atomicCAS(a.flag, 0, i + 1);
    const double LUki = ld_l2(a.data + i) / LUii;
    st_l2(a.data + i, LUki);
    for (int u = a.upd_ptr[i]; u < a.upd_ptr[i + 1]; ++u) {
      const int l = a.upd_l[u];
      st_l2(a.data + l, ld_l2(a.data + l) - LUki * ld_l2(a.data + a.upd_j[u]));
    }
  }
}

__device__ __forceinline__ void factor_row(const FactorArgs& a, int k) {
  const int r0 = a.rowptr[k], r1 = a.rowptr[k + 1], dk = a.diag[k];
  if (r1 - r0 > FACTOR_ROW_MAX) {
    factor_row_global(a, k);
    return;
  }
  // the row's own values: only this thread reads or writes them
  double rowv[FACTOR_ROW_MAX];
  for (int q = 0; q < r1 - r0; ++q) rowv[q] = ld_l2(a.data + r0 + q);
  for (int i = r0; i < dk; ++i) {
    const double LUii = ld_l2(a.data + a.diag[a.col[i]]);
    if (LUii == 0) atomicCAS(a.flag, 0, i + 1);
    const double LUki = rowv[i - r0] / LUii;
    rowv[i - r0] = LUki;
    const int u0 = a.upd_ptr[i], u1 = a.upd_ptr[i + 1];
    for (int ub = u0; ub < u1; ub += FACTOR_BATCH) {
      // values of earlier rows: independent loads issued together
      double dj[FACTOR_BATCH];
      int lo[FACTOR_BATCH];
#pragma unroll
      for (int q = 0; q < FACTOR_BATCH; ++q)
        if (ub + q < u1) {
          dj[q] = ld_l2(a.data + a.upd_j[ub + q]);
          lo[q] = a.upd_l[ub + q] - r0;
        }
#pragma unroll
      for (int q = 0; q < FACTOR_BATCH; ++q)
        if (ub + q < u1) rowv[lo[q]] = rowv[lo[q]] - LUki * dj[q];
    }
  }
  for (int q = 0; q < r1 - r0; ++q) st_l2(a.data + r0 + q, rowv[q]);
}

__global__ void __launch_bounds__(512) k_factor_cluster(FactorArgs a) {
  cg::cluster_group cluster = cg::this_cluster();
  const int nthreads = (int)cluster.num_blocks() * blockDim.x;
  const int t = (int)cluster.block_rank() * blockDim.x + threadIdx.x;
  for (int l = 0; l < a.nlev; ++l) {
    const int r0 = a.level_slices[l] * 32, r1 = a.level_slices[l + 1] * 32;
    for (int slot = r0 + t; slot < r1; slot += nthreads) {
      const int k = a.row[slot];
      if (k >= 0) factor_row(a, k);
    }
    cluster.sync();
  }
}

__global__ void k_factor_level(FactorArgs a, int l) {
  const int slot = a.level_slices[l] * 32 + blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= a.level_slices[l + 1] * 32) return;
  const int k = a.row[slot];
  if (k >= 0) factor_row(a, k);
}

template <typename T>
__global__ void k_plan_gather(int64_t size, const int* __restrict__ src, const double* __restrict__ v,
                              T* __restrict__ out) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= size) return;
  int s = src[q];
  out[q] = s >= 0 ? (T)v[s] : (T)0;
}

__global__ void k_copy(int64_t n, const double* __restrict__ a, double* __restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

__global__ void k_invdiag(int n, const int* __restrict__ diag, const double* __restrict__ val, double* inv,
                          float* invf, int* flag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double d = diag[i] >= 0 ? val[diag[i]] : 0.0;
  if (d == 0) atomicCAS(flag, 0, i + 1);
  inv[i] = 1 / d;
  invf[i] = (float)(1 / d);
}

template <typename T>
__global__ void k_diag_apply(int n, const T* __restrict__ inv, const T* __restrict__ b, T* __restrict__ x,
                             const int* active) {
  if (active && *active != 0) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = b[i] * inv[i];
}

// ------------------------------------------------------- ring planning ----
// Host form of a RingPlan (see k_sweep_ring).  Rows belong to CTAs in
// contiguous blocks (owner = row * C / n); each dependency level is split
// into plan levels of at most W * 32 rows per CTA.
struct HostRing {
  int C = 0, nlev = 0, R = 0, slack = 0, maxlen = 0;
  std::vector<int> slice_base, row, len, ridx, src, diag_src, expect;
  std::vector<unsigned short> pmask, nbr;
};

// Largest padded slot count accepted for a ring plan: levels hold
// RING_SLOT slots whether or not they are full, so a pattern with very many
// narrow levels (a tridiagonal matrix) walks with the plain cluster kernels.
static int64_t ring_slot_budget(int n) { return 8 * (int64_t)n + (int64_t)8 * 1024 * 1024; }

// Builds the ring schedule of one sweep.  entries: 0 strictly lower part, 1
// strictly upper part; upper_levels: dependencies on higher rows.  Returns
// false when no schedule exists within the shared-memory and slot limits.
static bool plan_ring(int n, const std::vector<int>& rp, const std::vector<int>& cl, const std::vector<int>& dg,
                      bool upper_levels, int entries, int C, size_t max_smem, HostRing& H) {
  if (n <= 0 || C < 1 || C > RING_MAX_CTAS || RING_SLICES % C) return false;
  const int W = RING_SLICES / C, cap = W * 32;
  auto ent = [&](int r, int& q0, int& q1) {
    if (entries == 0) {
      q0 = rp[r];
      q1 = dg[r];
    } else {
      q0 = dg[r] + 1;
      q1 = rp[r + 1];
    }
  };
  std::vector<int> lev(n, 0);
  if (!upper_levels) {
    for (int i = 0; i < n; ++i) {
      int L = 0, q0, q1;
      ent(i, q0, q1);
      for (int q = q0; q < q1; ++q) L = std::max(L, lev[cl[q]] + 1);
      lev[i] = L;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int L = 0, q0, q1;
      ent(i, q0, q1);
      for (int q = q0; q < q1; ++q) L = std::max(L, lev[cl[q]] + 1);
      lev[i] = L;
    }
  }
  int ndep = 0;
  for (int i = 0; i < n; ++i) ndep = std::max(ndep, lev[i] + 1);
  auto owner = [&](int r) { return (int)((int64_t)r * C / n); };
  // rows per (dependency level, CTA) and the plan levels of each dependency level
  std::vector<int> cnt((size_t)ndep * C, 0);
  for (int i = 0; i < n; ++i) cnt[(size_t)lev[i] * C + owner(i)]++;
  std::vector<int> pl0(ndep + 1, 0);
  for (int L = 0; L < ndep; ++L) {
    int sub = 1;
    for (int c = 0; c < C; ++c) sub = std::max(sub, (cnt[(size_t)L * C + c] + cap - 1) / cap);
    pl0[L + 1] = pl0[L] + sub;
  }
  const int nlev = pl0[ndep];
  if ((int64_t)nlev * RING_SLOT > ring_slot_budget(n)) return false;
  std::vector<int> plev(n), ppos(n);
  std::fill(cnt.begin(), cnt.end(), 0);
  for (int i = 0; i < n; ++i) {  // ascending rows within a CTA's level
    const int c = owner(i);
    const int k = cnt[(size_t)lev[i] * C + c]++;
    plev[i] = pl0[lev[i]] + k / cap;
    ppos[i] = c * cap + k % cap;
  }
  int look = 0;
  for (int i = 0; i < n; ++i) {
    int q0, q1;
    ent(i, q0, q1);
    for (int q = q0; q < q1; ++q) look = std::max(look, plev[i] - plev[cl[q]]);
  }
  // the deepest ring that fits gives the most slack (at most the lookback: R >= 2 S + 2)
  if (ring_smem_bytes<double>(look + 2) > max_smem) return false;
  int S = 0;
  while (S < look && ring_smem_bytes<double>(look + 3 + S) <= max_smem) ++S;
  const int R = look + 2 + S;
  const size_t nslot = (size_t)nlev * RING_SLOT, nslice = (size_t)nlev * RING_SLICES;
  H.C = C;
  H.nlev = nlev;
  H.R = R;
  H.slack = S;
  H.row.assign(nslot, -1);
  H.len.assign(nslot, 0);
  H.diag_src.assign(nslot, -1);
  std::vector<int> width(nslice, 0);
  for (int i = 0; i < n; ++i) {
    int q0, q1;
    ent(i, q0, q1);
    const size_t slot = (size_t)plev[i] * RING_SLOT + ppos[i];
    H.row[slot] = i;
    H.len[slot] = q1 - q0;
    H.maxlen = std::max(H.maxlen, q1 - q0);
    H.diag_src[slot] = dg[i];
    width[slot / 32] = std::max(width[slot / 32], q1 - q0);
  }
  H.slice_base.assign(nslice + 1, 0);
  int64_t pos = 0;
  for (size_t s = 0; s < nslice; ++s) {
    H.slice_base[s] = (int)pos;
    pos += (int64_t)width[s] * 32;
    if (pos > INT32_MAX) return false;
  }
  H.slice_base[nslice] = (int)pos;
  H.ridx.assign(std::max<int64_t>(pos, 1), 0);
  H.src.assign(std::max<int64_t>(pos, 1), -1);
  // which CTAs read each row's value
  std::vector<unsigned short> mask(n, 0);
  for (int i = 0; i < n; ++i) {
    int q0, q1;
    ent(i, q0, q1);
    const size_t slot = (size_t)plev[i] * RING_SLOT + ppos[i];
    const int64_t b = H.slice_base[slot / 32] + (int64_t)(slot % 32);
    for (int q = q0, k = 0; q < q1; ++q, ++k) {
      const int j = cl[q];
      H.src[b + 32 * k] = q;
      H.ridx[b + 32 * k] = (plev[j] % R) * RING_SLOT + ppos[j];
      if (owner(j) != owner(i)) mask[j] |= (unsigned short)(1u << owner(i));
    }
  }
  H.pmask.assign(nslot, 0);
  H.expect.assign((size_t)nlev * C, 0);
  H.nbr.assign(C, 0);
  for (size_t s0 = 0; s0 < nslot; s0 += 2) {
    const int r0 = H.row[s0], r1 = H.row[s0 + 1];
    if (r0 < 0) continue;
    const unsigned short m = (unsigned short)(mask[r0] | (r1 >= 0 ? mask[r1] : 0));
    H.pmask[s0] = m;
    const int l = (int)(s0 / RING_SLOT), c = owner(r0);
    H.nbr[c] |= m;
    for (int t = 0; t < C; ++t)
      if (m >> t & 1) H.expect[(size_t)l * C + t] += 2;
  }
  for (int c = 0; c < C; ++c)
    for (int t = 0; t < C; ++t)
      if (H.nbr[c] >> t & 1) H.nbr[t] |= (unsigned short)(1u << c);
  return true;
}

// Independent check of a ring schedule against the matrix: every row is
// placed once, every slot and entry index stays inside its arrays, every
// operand of a row lies in an earlier level within the ring's reach and is
// either the CTA's own value or pushed to it, and the expected counts equal
// the values pushed.  Returns an empty string when the schedule is sound.
static std::string check_ring(int n, const std::vector<int>& rp, const std::vector<int>& cl,
                              const std::vector<int>& dg, int entries, const HostRing& H) {
  const int C = H.C, R = H.R, W = RING_SLICES / C;
  const size_t nslot = (size_t)H.nlev * RING_SLOT;
  if (H.row.size() != nslot || H.len.size() != nslot || H.pmask.size() != nslot) return "slot arrays";
  if (H.slice_base.size() != (size_t)H.nlev * RING_SLICES + 1) return "slice offsets";
  if (R < 2 || ring_smem_bytes<double>(R) > RING_SMEM_MAX) return "ring depth";
  if (H.slack < 0 || R < 2 * H.slack + 2) return "slack";
  const int64_t nent = H.slice_base.back();
  std::vector<int> plev(n, -1), ppos(n, -1);
  auto owner = [&](int r) { return (int)((int64_t)r * C / n); };
  for (size_t s = 0; s < nslot; ++s) {
    const int r = H.row[s];
    if (r < -1 || r >= n) return "row id out of range";
    if (r < 0) {
      if (H.pmask[s]) return "mask on an empty slot";
      continue;
    }
    if (plev[r] >= 0) return "row placed twice";
    plev[r] = (int)(s / RING_SLOT);
    ppos[r] = (int)(s % RING_SLOT);
    if (ppos[r] / (W * 32) != owner(r)) return "row outside its CTA's slots";
    if ((s & 1) && H.row[s - 1] < 0) return "odd lane active without its even lane";
  }
  for (int i = 0; i < n; ++i)
    if (plev[i] < 0) return "row missing";
  std::vector<int> got((size_t)H.nlev * C, 0);
  for (size_t s = 0; s < nslot; ++s) {
    const int r = H.row[s];
    if (r < 0) continue;
    const int q0 = entries == 0 ? rp[r] : dg[r] + 1, q1 = entries == 0 ? dg[r] : rp[r + 1];
    if (H.len[s] != q1 - q0) return "row length";
    const size_t sl = s / 32;
    const int64_t w = (int64_t)(H.slice_base[sl + 1] - H.slice_base[sl]) / 32;
    if (H.len[s] > w) return "row longer than its slice";
    for (int k = 0; k < H.len[s]; ++k) {
      const int64_t e = H.slice_base[sl] + (int64_t)(s % 32) + 32 * (int64_t)k;
      if (e < 0 || e >= nent) return "entry index out of range";
      const int j = cl[q0 + k];
      if (H.src[e] != q0 + k) return "entry source";
      if (H.ridx[e] < 0 || H.ridx[e] >= R * RING_SLOT) return "ring index out of range";
      if (H.ridx[e] != (plev[j] % R) * RING_SLOT + ppos[j]) return "ring index";
      if (plev[j] >= plev[r] || plev[r] - plev[j] > R - 2 - H.slack) return "operand outside the ring's reach";
      if (owner(j) != owner(r)) {
        const size_t sj = (size_t)plev[j] * RING_SLOT + ppos[j];
        if (!(H.pmask[sj & ~(size_t)1] >> owner(r) & 1)) return "operand not pushed to its reader";
      }
    }
    if (!(s & 1)) {
      const unsigned m = H.pmask[s];
      if (m >> owner(r) & 1) return "value pushed to its own CTA";
      if (m & ~H.nbr[owner(r)]) return "push target is not a neighbour";
      for (int t = 0; t < C; ++t)
        if (m >> t & 1) got[(size_t)(s / RING_SLOT) * C + t] += 2;
    }
  }
  if (got != H.expect) return "expected counts";
  for (int c = 0; c < C; ++c) {
    if (H.nbr[c] >> c & 1) return "neighbour of itself";
    for (int t = 0; t < C; ++t)
      if ((H.nbr[c] >> t & 1) != (H.nbr[t] >> c & 1)) return "neighbour masks not symmetric";
  }
  return "";
}

// ------------------------------------------------------------ planning ----
// entries: 0 lower part, 1 upper part, 2 full row without the diagonal.
// upper_levels: schedule by dependencies on higher rows (backward sweeps).
static void build_plan(Csr& A, SweepPlan& P, bool upper_levels, int entries, bool with_diag) {
  const int n = A.n;
  const auto& rp = A.h_rowptr;
  const auto& cl = A.h_col;
  const auto& dg = A.h_diag;
  std::vector<int> lev(n, 0);
  if (!upper_levels) {
    for (int i = 0; i < n; ++i) {
      int L = 0;
      for (int q = rp[i]; q < rp[i + 1] && cl[q] < i; ++q) L = std::max(L, lev[cl[q]] + 1);
      lev[i] = L;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int L = 0;
      for (int q = rp[i + 1] - 1; q >= rp[i] && cl[q] > i; --q) L = std::max(L, lev[cl[q]] + 1);
      lev[i] = L;
    }
  }
  int nlev = 0;
  for (int i = 0; i < n; ++i) nlev = std::max(nlev, lev[i] + 1);
  std::vector<int> cnt(nlev + 1, 0);
  for (int i = 0; i < n; ++i) cnt[lev[i] + 1]++;
  for (int l = 0; l < nlev; ++l) cnt[l + 1] += cnt[l];
  std::vector<int> order(n), fill(cnt.begin(), cnt.end() - 1);
  for (int i = 0; i < n; ++i) order[fill[lev[i]]++] = i;  // ascending row within a level
  // slices per level
  std::vector<int> level_slices(nlev + 1, 0);
  for (int l = 0; l < nlev; ++l) {
    int rows = cnt[l + 1] - cnt[l];
    level_slices[l + 1] = level_slices[l] + (rows + 31) / 32;
    P.max_rows_per_level = std::max(P.max_rows_per_level, rows);
  }
  const int ns = level_slices[nlev];
  std::vector<int> row((size_t)ns * 32, -1), len((size_t)ns * 32, 0), base(ns + 1, 0), width(ns, 0);
  auto row_entries = [&](int r, int& b0, int& b1, int& c0, int& c1) {
    // returns up to two ranges [b0,b1) and [c0,c1) of CSR positions
    b0 = b1 = c0 = c1 = rp[r];
    int d = dg[r];
    if (entries == 0) {
      b0 = rp[r];
      b1 = d;
    } else if (entries == 1) {
      b0 = d + 1;
      b1 = rp[r + 1];
    } else {
      b0 = rp[r];
      b1 = d;
      c0 = d + 1;
      c1 = rp[r + 1];
    }
  };
  for (int l = 0; l < nlev; ++l) {
    for (int t = 0; t < cnt[l + 1] - cnt[l]; ++t) {
      int s = level_slices[l] + t / 32, lane = t % 32;
      int r = order[cnt[l] + t];
      row[(size_t)s * 32 + lane] = r;
      int b0, b1, c0, c1;
      row_entries(r, b0, b1, c0, c1);
      int L = (b1 - b0) + (c1 - c0);
      len[(size_t)s * 32 + lane] = L;
      width[s] = std::max(width[s], L);
    }
  }
  int64_t pos = 0;
  for (int s = 0; s < ns; ++s) {
    base[s] = (int)pos;
    pos += (int64_t)width[s] * 32;
  }
  base[ns] = (int)pos;
  if (pos > INT32_MAX) throw Error(RSG_UNSUPPORTED, "matrix too large for 32-bit sweep offsets");
  std::vector<int> col(std::max<int64_t>(pos, 1), 0), src(std::max<int64_t>(pos, 1), -1);
  std::vector<int> dsrc((size_t)ns * 32, -1);
  for (int s = 0; s < ns; ++s)
    for (int lane = 0; lane < 32; ++lane) {
      int r = row[(size_t)s * 32 + lane];
      if (r < 0) continue;
      dsrc[(size_t)s * 32 + lane] = dg[r];
      int b0, b1, c0, c1;
      row_entries(r, b0, b1, c0, c1);
      int k = 0;
      for (int q = b0; q < b1; ++q, ++k) {
        col[base[s] + 32 * k + lane] = cl[q];
        src[base[s] + 32 * k + lane] = q;
      }
      for (int q = c0; q < c1; ++q, ++k) {
        col[base[s] + 32 * k + lane] = cl[q];
        src[base[s] + 32 * k + lane] = q;
      }
    }
  // push-ring schedules (lower or upper ILU parts only), for both cluster
  // shapes unless RSG_RING_CTAS fixes one
  HostRing H[2];
  bool ring[2] = {false, false};
  for (int v = 0; v < 2; ++v) {
    const int C = v == 0 ? 16 : 8;
    if (ring_ctas() != 0 && ring_ctas() != C) continue;
    ring[v] = entries != 2 && plan_ring(n, rp, cl, dg, upper_levels, entries, C, RING_SMEM_MAX, H[v]);
  }
  Context& ctx = *A.ctx;
  P.nlev = nlev;
  P.nslices = ns;
  P.h_level_slices = level_slices;
  P.level_slices.resize(nlev + 1);
  P.slice_base.resize(ns + 1);
  P.row.resize((size_t)ns * 32 + 1);
  P.len.resize((size_t)ns * 32 + 1);
  P.col.resize(col.size());
  P.src.resize(src.size());
  P.val.resize(col.size());
  P.valf.resize(col.size());
  auto up = [&](auto& dst, const auto& v) {
    RSG_CUDA(cudaMemcpyAsync(dst.get(), v.data(), sizeof(v[0]) * v.size(), cudaMemcpyHostToDevice, ctx.stream));
  };
  up(P.level_slices, level_slices);
  up(P.slice_base, base);
  up(P.row, row);
  up(P.len, len);
  up(P.col, col);
  up(P.src, src);
  for (int v = 0; v < 2; ++v) {
    RingPlan& G = P.rings[v];
    G.R = 0;
    if (!ring[v]) continue;
    const HostRing& Hv = H[v];
    G.C = Hv.C;
    G.nlev = Hv.nlev;
    G.R = Hv.R;
    G.slack = Hv.slack;
    G.maxlen = Hv.maxlen;
    G.slice_base.resize(Hv.slice_base.size());
    G.row.resize(Hv.row.size());
    G.len.resize(Hv.len.size());
    G.ridx.resize(Hv.ridx.size());
    G.src.resize(Hv.src.size());
    G.pmask.resize(Hv.pmask.size());
    G.expect.resize(Hv.expect.size());
    G.nbr.resize(Hv.nbr.size());
    G.val.resize(Hv.src.size());
    G.valf.resize(Hv.src.size());
    up(G.slice_base, Hv.slice_base);
    up(G.row, Hv.row);
    up(G.len, Hv.len);
    up(G.ridx, Hv.ridx);
    up(G.src, Hv.src);
    up(G.pmask, Hv.pmask);
    up(G.expect, Hv.expect);
    up(G.nbr, Hv.nbr);
    if (with_diag) {
      G.diag_src.resize(Hv.diag_src.size());
      G.diag.resize(Hv.diag_src.size());
      G.diagf.resize(Hv.diag_src.size());
      up(G.diag_src, Hv.diag_src);
    }
  }
  // until the autotuner has timed them: 16 CTAs where that schedule exists
  P.pick[0] = P.pick[1] = P.rings[0].R ? 0 : 1;
  P.tuned = false;
  if (with_diag) {
    P.diag_src.resize(dsrc.size());
    P.diag.resize(dsrc.size());
    P.diagf.resize(dsrc.size());
    up(P.diag_src, dsrc);
  }
  ctx.sync();
}

template <typename T>
__global__ void k_fill_one(int n, T* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = T(1);
}

static void plan_values(Context& ctx, SweepPlan& P, const double* csr_vals, bool with_diag, bool f32) {
  int64_t size = (int64_t)P.src.size();
  RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<double>, blocks_for(size, 256), 256, 0, size, P.src.get(), csr_vals,
             P.val.get());
  if (f32)
    RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<float>, blocks_for(size, 256), 256, 0, size, P.src.get(), csr_vals,
               P.valf.get());
  if (with_diag) {
    int64_t ds = (int64_t)P.diag_src.size();
    RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<double>, blocks_for(ds, 256), 256, 0, ds, P.diag_src.get(),
               csr_vals, P.diag.get());
    if (f32)
      RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<float>, blocks_for(ds, 256), 256, 0, ds, P.diag_src.get(),
                 csr_vals, P.diagf.get());
  }
  for (RingPlan& G : P.rings) {
  if (!G.R) continue;
  const int64_t gs = (int64_t)G.src.size();
  RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<double>, blocks_for(gs, 256), 256, 0, gs, G.src.get(), csr_vals,
             G.val.get());
  if (f32)
    RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<float>, blocks_for(gs, 256), 256, 0, gs, G.src.get(), csr_vals,
               G.valf.get());
  if (with_diag) {
    const int64_t ds = (int64_t)G.diag_src.size();
    RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<double>, blocks_for(ds, 256), 256, 0, ds, G.diag_src.get(),
               csr_vals, G.diag.get());
    if (f32)
      RSG_LAUNCH(ctx, "plan_gather", k_plan_gather<float>, blocks_for(ds, 256), 256, 0, ds, G.diag_src.get(),
                 csr_vals, G.diagf.get());
  }
}
}

// Cluster launch of a level walk; falls back to one launch per level when
// clusters of the requested size cannot be scheduled.
// Probes run once per process; contexts driven from several host threads
// (ensembles) take the lock for them.
static std::mutex g_probe_mu;
static std::atomic<int> g_cluster_ok{-1};  // probed once per process

template <typename Kernel, typename Args>
static bool launch_cluster(Context& ctx, const char* name, Kernel kern, const Args& args, int threads = 512) {
  std::atomic<int>& cluster_ok = g_cluster_ok;
  std::unique_lock<std::mutex> lk(g_probe_mu, std::defer_lock);
  if (cluster_ok < 0) lk.lock();
  if (cluster_ok < 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctx.cluster_size);
    cfg.blockDim = dim3(threads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctx.cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, (const void*)kern, &cfg);
    cluster_ok = (e == cudaSuccess && nclusters >= 1) ? 1 : 0;
    cudaGetLastError();
  }
  if (lk.owns_lock()) lk.unlock();
  if (!cluster_ok) return false;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctx.cluster_size);
  cfg.blockDim = dim3(threads);
  cfg.stream = ctx.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ctx.cluster_size;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  LaunchScope scope(ctx, name);
  RSG_CUDA(cudaLaunchKernelEx(&cfg, kern, args));
  return true;
}

// Push-ring launch: one cluster of the plan's CTA count with the ring and its
// mbarriers in dynamic shared memory.  The plan is built for 16 CTAs of 4
// warps (RSG_RING_CTAS=8 selects 8 CTAs of 8 warps); RSG_SWEEP=pipelined
// switches the ring off.  Returns false when the plan has no ring schedule
// or no such cluster can be scheduled.
static std::atomic<bool> g_ring_used{false};

template <typename Kernel>
static bool ring_schedulable(Kernel kern, int ctas, size_t smem) {
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (ctas > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(RING_SLICES / ctas * 32);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, (const void*)kern, &cfg);
  cudaGetLastError();
  return e == cudaSuccess && nclusters >= 1;
}

// MAXW: the entries of a row held in registers.  Every unrolled step costs
// issue slots whether its lanes are active or not, so the kernel is built
// for 13 entries (the 27-point stencil's triangles) and for 16; longer rows
// read their remaining entries from memory.
template <int KIND, typename T, int CTAS, int MAXW, bool FMA>
static bool launch_ring_n(Context& ctx, const char* name, const RingPlan& G, const RingVals<T>& a, size_t smem) {
  auto kern = k_sweep_ring<KIND, T, MAXW, CTAS, FMA>;
  static std::atomic<int> ok{0};  // per instantiation: 0 not probed, 1 schedulable, -1 not
  if (!ok) {
    std::lock_guard<std::mutex> lk(g_probe_mu);
    if (!ok) ok = ring_schedulable(kern, CTAS, RING_SMEM_MAX) ? 1 : -1;
  }
  if (ok < 0) return false;
  RingArgs g{G.nlev,        G.R,           G.slack,       G.slice_base.get(), G.row.get(), G.len.get(),
             G.ridx.get(), G.pmask.get(), G.expect.get(), G.nbr.get(),       ctx.dev_err.get()};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CTAS);
  cfg.blockDim = dim3(RING_SLICES / CTAS * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = ctx.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CTAS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  LaunchScope scope(ctx, name);
  RSG_CUDA(cudaLaunchKernelEx(&cfg, kern, g, a));
  g_ring_used = true;
  return true;
}

template <typename T>
struct RingPick;
template <>
struct RingPick<double> {
  static const double* val(const RingPlan& G) { return G.val.get(); }
  static const double* diag(const RingPlan& G) { return G.diag.get(); }
};
template <>
struct RingPick<float> {
  static const float* val(const RingPlan& G) { return G.valf.get(); }
  static const float* diag(const RingPlan& G) { return G.diagf.get(); }
};

template <int KIND, typename T, bool FMA>
static bool launch_ring(Context& ctx, const char* name, const SweepPlan& P, const T* val, const T* diag, const T* b,
                        T* x, const int* active) {
  const RingPlan& G = P.ring(sizeof(T) == 4 ? 1 : 0);
  if (!ring_enabled() || !G.R) return false;
  const size_t smem = ring_smem_bytes<T>(G.R);
  if (smem > RING_SMEM_MAX) return false;
  const RingVals<T> a{val, diag, b, x, active};
  const bool narrow = G.maxlen <= 13;
  if (G.C == 16)
    return narrow ? launch_ring_n<KIND, T, 16, 13, FMA>(ctx, name, G, a, smem)
                  : launch_ring_n<KIND, T, 16, 16, FMA>(ctx, name, G, a, smem);
  if (G.C == 8)
    return narrow ? launch_ring_n<KIND, T, 8, 13, FMA>(ctx, name, G, a, smem)
                  : launch_ring_n<KIND, T, 8, 16, FMA>(ctx, name, G, a, smem);
  return false;
}

// FMA: the ring walk sums each row with fused multiply-adds (the Krylov
// solvers' applies); otherwise every path rounds as MTJ does.
template <int KIND, typename T, bool FMA = false>
static void run_sweep(Context& ctx, const char* name, const SweepPlan& P, const T* val, const T* diag, const T* b,
                      T* x, T* xx, T omega, const int* active) {
  SweepArgs<T> a{P.nlev, P.level_slices.get(), P.slice_base.get(), P.row.get(), P.len.get(), P.col.get(), val, diag,
                 b, x, xx, omega, active};
  if constexpr (KIND == SW_ILU_LOWER || KIND == SW_ILU_UPPER) {
    const RingPlan& G = P.ring(sizeof(T) == 4 ? 1 : 0);
    const bool ring = launch_ring<KIND, T, FMA>(ctx, name, P, RingPick<T>::val(G),
                                                KIND == SW_ILU_UPPER ? RingPick<T>::diag(G) : nullptr, b, x, active);
    if (ring) return;
  }
  if ((KIND == SW_ILU_LOWER || KIND == SW_ILU_UPPER) && P.nlev <= SWEEP_MAX_LEVELS) {
    if (launch_cluster(ctx, name, k_sweep_pipelined<KIND, T, 16>, a, 256)) return;
  } else if (launch_cluster(ctx, name, k_sweep_cluster<KIND, T>, a))
    return;
  for (int l = 0; l < P.nlev; ++l) {
    int slices = P.h_level_slices[l + 1] - P.h_level_slices[l];
    RSG_LAUNCH(ctx, name, (k_sweep_level<KIND, T>), blocks_for(slices, 8), 256, 0, a, l);
  }
}

// ------------------------------------------------------------------ ILU ----
struct ILUPrecond : Precond {
  Context* ctx;
  Csr* A = nullptr;
  SweepPlan Lp, Up;
  DeviceBuffer<double> LU, y;
  DeviceBuffer<float> yf;
  DeviceBuffer<int> flag, upd_ptr, upd_l, upd_j;
  const int* pattern_id = nullptr;
  explicit ILUPrecond(Context* c) : ctx(c) {}

  void analyse(Csr& M) {
    const auto& rp = M.h_rowptr;
    const auto& cl = M.h_col;
    for (int k = 0; k < M.n; ++k)
      if (M.h_diag[k] < 0)
        throw Error(RSG_MISSING_DIAGONAL, "Missing diagonal entry on row " + std::to_string(k + 1));
    // ILU.java:113-120 reads colind[l] one past the end of row k when the
    // scan of row k runs off its end; that read can update row k+1 or run
    // off the array.  Such patterns are rejected rather than reproduced.
    for (int k = 1; k < M.n; ++k) {
      const int r1 = rp[k + 1];
      const int maxc = cl[r1 - 1];
      for (int i = rp[k]; i < M.h_diag[k]; ++i) {
        int index = cl[i];
        if (cl[rp[index + 1] - 1] <= maxc) continue;
        for (int j = M.h_diag[index] + 1; j < rp[index + 1]; ++j)
          if (cl[j] > maxc) {
            if (r1 >= M.nnz || cl[r1] == cl[j])
              throw Error(RSG_UNSUPPORTED, "ILU(0) pattern reaches past the end of row " + std::to_string(k + 1));
          }
      }
    }
    // elimination program (see FactorArgs)
    {
      std::vector<int> uptr(M.nnz + 1, 0), ul, uj;
      ul.reserve((size_t)M.nnz * 4);
      uj.reserve((size_t)M.nnz * 4);
      for (int k = 0; k < M.n; ++k) {
        const int r1 = rp[k + 1];
        for (int i = rp[k]; i < M.h_diag[k]; ++i) {
          const int index = cl[i];
          int l = rp[k] + 1;
          int cnt = 0;
          for (int j = M.h_diag[index] + 1; j < rp[index + 1]; ++j) {
            while (l < r1 && cl[l] < cl[j]) l++;
            if (l < r1 && cl[l] == cl[j]) {
              ul.push_back(l);
              uj.push_back(j);
              cnt++;
            }
          }
          uptr[i + 1] = cnt;
        }
      }
      for (int q = 0; q < M.nnz; ++q) uptr[q + 1] += uptr[q];
      if (ul.size() > (size_t)INT32_MAX) throw Error(RSG_UNSUPPORTED, "ILU elimination program too large");
      if (ul.empty()) {
        ul.push_back(0);
        uj.push_back(0);
      }
      upd_ptr.resize(M.nnz + 1);
      upd_l.resize(ul.size());
      upd_j.resize(uj.size());
      RSG_CUDA(cudaMemcpyAsync(upd_ptr.get(), uptr.data(), sizeof(int) * uptr.size(), cudaMemcpyHostToDevice,
                               ctx->stream));
      RSG_CUDA(cudaMemcpyAsync(upd_l.get(), ul.data(), sizeof(int) * ul.size(), cudaMemcpyHostToDevice, ctx->stream));
      RSG_CUDA(cudaMemcpyAsync(upd_j.get(), uj.data(), sizeof(int) * uj.size(), cudaMemcpyHostToDevice, ctx->stream));
      ctx->sync();
    }
    build_plan(M, Lp, false, 0, false);
    build_plan(M, Up, true, 1, true);
    LU.resize(std::max(M.nnz, 1));
    y.resize(M.n);
    yf.resize(M.n);
    flag.resize(1);
  }

  void setup(Csr& M) override {
    if (A != &M || pattern_id != M.rowptr.get()) {
      analyse(M);
      A = &M;
      pattern_id = M.rowptr.get();
    }
    // LU.set(A) then factor() (ILU.java:80-125)
    RSG_LAUNCH(*ctx, "ilu_copy", k_copy, blocks_for(M.nnz, 256), 256, 0, (int64_t)M.nnz, M.val.get(), LU.get());
    RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), ctx->stream));
    FactorArgs fa{Lp.nlev,      Lp.level_slices.get(), Lp.row.get(), M.rowptr.get(), M.col.get(), M.diag.get(),
                  upd_ptr.get(), upd_l.get(),           upd_j.get(),  LU.get(),       flag.get()};
    if (!launch_cluster(*ctx, "ilu_factor", k_factor_cluster, fa)) {
      for (int l = 0; l < Lp.nlev; ++l) {
        int slots = (Lp.h_level_slices[l + 1] - Lp.h_level_slices[l]) * 32;
        RSG_LAUNCH(*ctx, "ilu_factor", k_factor_level, blocks_for(slots, 256), 256, 0, fa, l);
      }
    }
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (h) throw Error(RSG_ZERO_PIVOT, "Zero pivot encountered on row " + std::to_string(h));
    plan_values(*ctx, Lp, LU.get(), false, true);
    plan_values(*ctx, Up, LU.get(), true, true);
    if (!Lp.tuned || !Up.tuned) tune_walks();
  }

  // Walk autotuner: the first setup on a pattern times each sweep's ring
  // schedules (16 CTAs of 4 warps, 8 CTAs of 8 warps) on the factor values,
  // for the FP64 and the FP32 walks as the solvers run them (FP64 with fused
  // multiply-adds), and keeps the faster per sweep and precision.  Every schedule sums each row in CSR order, so the choice
  // never changes a result bit.  force_ctas (rsg_solver_set_walk_shape)
  // replaces the timing by a fixed shape.
  int force_ctas = 0;
  void tune_walks() {
    const int n = A->n;
    DeviceBuffer<double> bd(n), xd(n);
    DeviceBuffer<float> bf(n), xf(n);
    RSG_LAUNCH(*ctx, "tune_fill", k_fill_one<double>, blocks_for(n, 256), 256, 0, n, bd.get());
    RSG_LAUNCH(*ctx, "tune_fill", k_fill_one<float>, blocks_for(n, 256), 256, 0, n, bf.get());
    cudaEvent_t e0, e1;
    RSG_CUDA(cudaEventCreate(&e0));
    RSG_CUDA(cudaEventCreate(&e1));
    auto time_ms = [&](auto&& run) {
      run();  // warm-up
      RSG_CUDA(cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < 3; ++r) run();
      RSG_CUDA(cudaEventRecord(e1, ctx->stream));
      RSG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      RSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      return ms;
    };
    for (SweepPlan* P : {&Lp, &Up}) {
      const bool lower = P == &Lp;
      for (int prec = 0; prec < 2; ++prec) {
        int best = P->pick[prec];
        float best_ms = 1e30f;
        for (int v = 0; v < 2; ++v) {
          if (!P->rings[v].R) continue;
          if (force_ctas && P->rings[v].C != force_ctas) continue;
          P->pick[prec] = v;
          float ms;
          if (prec == 0) {
            ms = time_ms([&] {
              if (lower)
                run_sweep<SW_ILU_LOWER, double, true>(*ctx, "ilu_tune", Lp, Lp.val.get(), nullptr, bd.get(), xd.get(),
                                                      nullptr, 0.0, nullptr);
              else
                run_sweep<SW_ILU_UPPER, double, true>(*ctx, "ilu_tune", Up, Up.val.get(), Up.diag.get(), bd.get(),
                                                      xd.get(), nullptr, 0.0, nullptr);
            });
          } else {
            ms = time_ms([&] {
              if (lower)
                run_sweep<SW_ILU_LOWER, float, true>(*ctx, "ilu_tune", Lp, Lp.valf.get(), nullptr, bf.get(), xf.get(),
                                                     nullptr, 0.0f, nullptr);
              else
                run_sweep<SW_ILU_UPPER, float, true>(*ctx, "ilu_tune", Up, Up.valf.get(), Up.diagf.get(), bf.get(),
                                                     xf.get(), nullptr, 0.0f, nullptr);
            });
          }
          if (ms < best_ms) {
            best_ms = ms;
            best = v;
          }
        }
        P->pick[prec] = best;
      }
      P->tuned = true;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->check_device_error();
  }

  // the Krylov solvers' applies: FP64 rows summed with fused multiply-adds
  void apply(const double* b, double* x, const int* active) override {
    // L.solve(b, y); U.solve(y, x)
    run_sweep<SW_ILU_LOWER, double, true>(*ctx, "ilu_lower", Lp, Lp.val.get(), nullptr, b, y.get(), nullptr, 0.0,
                                          active);
    run_sweep<SW_ILU_UPPER, double, true>(*ctx, "ilu_upper", Up, Up.val.get(), Up.diag.get(), y.get(), x, nullptr,
                                          0.0, active);
  }
  // Preconditioner.apply as MTJ rounds it (ILU.java:64-70)
  void apply_exact(const double* b, double* x) override {
    run_sweep<SW_ILU_LOWER, double>(*ctx, "ilu_lower", Lp, Lp.val.get(), nullptr, b, y.get(), nullptr, 0.0, nullptr);
    run_sweep<SW_ILU_UPPER, double>(*ctx, "ilu_upper", Up, Up.val.get(), Up.diag.get(), y.get(), x, nullptr, 0.0,
                                    nullptr);
  }
  void apply_f32(const float* b, float* x, const int* active) override {
    run_sweep<SW_ILU_LOWER, float, true>(*ctx, "ilu_lower_f32", Lp, Lp.valf.get(), nullptr, b, yf.get(), nullptr,
                                         0.0f, active);
    run_sweep<SW_ILU_UPPER, float, true>(*ctx, "ilu_upper_f32", Up, Up.valf.get(), Up.diagf.get(), yf.get(), x,
                                         nullptr, 0.0f, active);
  }
  void trans_apply(const double* b, double* x, const int* active) override;
};

// transApply (ILU.java:72-78) via column-oriented sweeps over the transpose;
// built lazily on first use.
struct TransPlan {
  Csr At;
  DeviceBuffer<int> tsrc;
  SweepPlan Lt, Ut;
  bool built = false;
};
static std::map<const ILUPrecond*, std::unique_ptr<TransPlan>> g_trans;

__global__ void k_gather_vals(int64_t n, const int* __restrict__ src, const double* __restrict__ v,
                              double* __restrict__ out) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = v[src[q]];
}

// U^T y = b: row i of U^T holds column i of U; y_i = (b_i - sum_{j<i} U_ji y_j) / U_ii.
// L^T x = y: x_i = y_i - sum_{j>i} L_ji x_j.
// The Java transSolve loops (UpperCompRowMatrix.java:69-90,
// UnitLowerCompRowMatrix.java:69-86) subtract the same products in row
// order of U and L; the transposed gather subtracts them in the same order.
void ILUPrecond::trans_apply(const double* b, double* x, const int* active) {
  auto& tp = g_trans[this];
  if (!tp) tp.reset(new TransPlan());
  TransPlan& T = *tp;
  Csr& M = *A;
  if (!T.built) {
    std::vector<int> tptr(M.n + 1, 0), tcol(M.nnz), tsrc(M.nnz);
    for (int q = 0; q < M.nnz; ++q) tptr[M.h_col[q] + 1]++;
    for (int c = 0; c < M.n; ++c) tptr[c + 1] += tptr[c];
    std::vector<int> fill(tptr.begin(), tptr.end() - 1);
    for (int r = 0; r < M.n; ++r)
      for (int q = M.h_rowptr[r]; q < M.h_rowptr[r + 1]; ++q) {
        int c = M.h_col[q];
        tcol[fill[c]] = r;
        tsrc[fill[c]] = q;
        fill[c]++;
      }
    T.At.build(ctx, M.n, M.nnz, tptr.data(), tcol.data());
    T.tsrc.resize(M.nnz);
    RSG_CUDA(cudaMemcpyAsync(T.tsrc.get(), tsrc.data(), sizeof(int) * M.nnz, cudaMemcpyHostToDevice, ctx->stream));
    ctx->sync();
    // U^T is lower triangular (its strictly lower part = U's strictly upper
    // part, transposed); L^T is upper triangular.
    build_plan(T.At, T.Ut, false, 0, true);
    build_plan(T.At, T.Lt, true, 1, false);
    T.built = true;
  }
  RSG_LAUNCH(*ctx, "ilu_trans_gather", k_gather_vals, blocks_for(M.nnz, 256), 256, 0, (int64_t)M.nnz, T.tsrc.get(),
             LU.get(), T.At.val.get());
  plan_values(*ctx, T.Ut, T.At.val.get(), true, false);
  plan_values(*ctx, T.Lt, T.At.val.get(), false, false);
  run_sweep<SW_ILU_UPPER, double>(*ctx, "ilu_trans_upper", T.Ut, T.Ut.val.get(), T.Ut.diag.get(), b, y.get(), nullptr,
                                  0.0, active);
  run_sweep<SW_ILU_LOWER, double>(*ctx, "ilu_trans_lower", T.Lt, T.Lt.val.get(), nullptr, y.get(), x, nullptr, 0.0,
                                  active);
}

// --------------------------------------------------------------- SSOR ----
struct SSORPrecond : Precond {
  Context* ctx;
  Csr* A = nullptr;
  const int* pattern_id = nullptr;
  SweepPlan Fp, Bp;
  DeviceBuffer<double> xx;
  DeviceBuffer<float> xxf;
  double omegaF = 1, omegaR = 1;
  bool reverse = true;
  explicit SSORPrecond(Context* c) : ctx(c) {}
  void setup(Csr& M) override {
    if (A != &M || pattern_id != M.rowptr.get()) {
      for (int k = 0; k < M.n; ++k)
        if (M.h_diag[k] < 0) throw Error(RSG_MISSING_DIAGONAL, "Missing diagonal on row " + std::to_string(k + 1));
      build_plan(M, Fp, false, 2, true);
      build_plan(M, Bp, true, 2, true);
      xx.resize(M.n);
      xxf.resize(M.n);
      A = &M;
      pattern_id = M.rowptr.get();
    }
    // FP32 copies too: the mixed-precision solver smooths its FP32 AMG levels with them
    plan_values(*ctx, Fp, M.val.get(), true, true);
    plan_values(*ctx, Bp, M.val.get(), true, true);
  }
  void apply_f32(const float* b, float* x, const int* active) override {
    run_sweep<SW_SSOR_FWD, float>(*ctx, "ssor_fwd_f32", Fp, Fp.valf.get(), Fp.diagf.get(), b, x, xxf.get(),
                                  (float)omegaF, active);
    if (!reverse) {
      RSG_CUDA(cudaMemcpyAsync(x, xxf.get(), sizeof(float) * A->n, cudaMemcpyDeviceToDevice, ctx->stream));
      return;
    }
    run_sweep<SW_SSOR_BWD, float>(*ctx, "ssor_bwd_f32", Bp, Bp.valf.get(), Bp.diagf.get(), b, x, xxf.get(),
                                  (float)omegaR, active);
  }
  void apply(const double* b, double* x, const int* active) override {
    // SSOR.java:143-194; x holds the starting iterate
    run_sweep<SW_SSOR_FWD, double>(*ctx, "ssor_fwd", Fp, Fp.val.get(), Fp.diag.get(), b, x, xx.get(), omegaF, active);
    if (!reverse) {
      RSG_LAUNCH(*ctx, "ssor_copy", k_copy, blocks_for(A->n, 256), 256, 0, (int64_t)A->n, xx.get(), x);
      return;
    }
    run_sweep<SW_SSOR_BWD, double>(*ctx, "ssor_bwd", Bp, Bp.val.get(), Bp.diag.get(), b, x, xx.get(), omegaR, active);
  }
  void trans_apply(const double* b, double* x, const int* active) override { apply(b, x, active); }
};

// ----------------------------------------------------------- diagonal ----
struct DiagPrecond : Precond {
  Context* ctx;
  int n = 0;
  DeviceBuffer<double> inv;
  DeviceBuffer<float> invf;
  DeviceBuffer<int> flag;
  explicit DiagPrecond(Context* c) : ctx(c) {}
  void setup(Csr& M) override {
    n = M.n;
    inv.resize(n);
    invf.resize(n);
    flag.resize(1);
    RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), ctx->stream));
    RSG_LAUNCH(*ctx, "diag_setup", k_invdiag, blocks_for(n, 256), 256, 0, n, M.diag.get(), M.val.get(), inv.get(),
               invf.get(), flag.get());
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (h) throw Error(RSG_ZERO_PIVOT, "Zero diagonal on row " + std::to_string(h));
  }
  void apply(const double* b, double* x, const int* active) override {
    RSG_LAUNCH(*ctx, "diag_apply", k_diag_apply<double>, blocks_for(n, 256), 256, 0, n, inv.get(), b, x, active);
  }
  void apply_f32(const float* b, float* x, const int* active) override {
    RSG_LAUNCH(*ctx, "diag_apply_f32", k_diag_apply<float>, blocks_for(n, 256), 256, 0, n, invf.get(), b, x, active);
  }
  void trans_apply(const double* b, double* x, const int* active) override { apply(b, x, active); }
};

struct IdentityPrecond : Precond {
  Context* ctx;
  int n = 0;
  explicit IdentityPrecond(Context* c) : ctx(c) {}
  void setup(Csr& M) override { n = M.n; }
  void apply(const double* b, double* x, const int* active) override {
    RSG_LAUNCH(*ctx, "copy", k_copy, blocks_for(n, 256), 256, 0, (int64_t)n, b, x);
  }
  void apply_f32(const float* b, float* x, const int* active) override {
    RSG_CUDA(cudaMemcpyAsync(x, b, sizeof(float) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  void trans_apply(const double* b, double* x, const int* active) override { apply(b, x, active); }
};

std::unique_ptr<Precond> make_precond(Context* ctx, int kind) {
  switch (kind) {
    case RSG_PC_NONE: return std::unique_ptr<Precond>(new IdentityPrecond(ctx));
    case RSG_PC_DIAGONAL: return std::unique_ptr<Precond>(new DiagPrecond(ctx));
    case RSG_PC_ILU: return std::unique_ptr<Precond>(new ILUPrecond(ctx));
    case RSG_PC_SSOR: return std::unique_ptr<Precond>(new SSORPrecond(ctx));
    case RSG_PC_AMG: return make_amg(ctx);
  }
  throw Error(RSG_UNSUPPORTED, "preconditioner not implemented");
}

bool ilu_walk_shape(Precond* p, int force, int* shapes) {
  auto* ilu = dynamic_cast<ILUPrecond*>(p);
  if (!ilu) return false;
  if (force >= 0) {
    ilu->force_ctas = force;
    ilu->Lp.tuned = ilu->Up.tuned = false;  // the next setup re-tunes
  }
  if (shapes) {
    const SweepPlan* P[2] = {&ilu->Lp, &ilu->Up};
    for (int prec = 0; prec < 2; ++prec)
      for (int s = 0; s < 2; ++s) {
        const RingPlan& G = P[s]->ring(prec);
        shapes[prec * 2 + s] = G.R ? G.C : 0;
      }
  }
  return true;
}

bool ilu_ring_plans(Precond* p, int prefer, const RingPlan** lower, const RingPlan** upper) {
  auto* ilu = dynamic_cast<ILUPrecond*>(p);
  if (!ilu || !ilu->A) return false;
  for (int pass = 0; pass < 2; ++pass)
    for (int v = 0; v < 2; ++v)
      if (ilu->Lp.rings[v].R && ilu->Up.rings[v].R && (pass == 1 || ilu->Lp.rings[v].C == prefer)) {
        *lower = &ilu->Lp.rings[v];
        *upper = &ilu->Up.rings[v];
        return true;
      }
  return false;
}

void set_ssor_params(Precond* p, double wf, double wr, int reverse) {
  auto* s = dynamic_cast<SSORPrecond*>(p);
  if (!s) throw Error(RSG_BAD_ARG, "solver does not use SSOR");
  if (wf < 0 || wf > 2 || wr < 0 || wr > 2) throw Error(RSG_BAD_ARG, "omega must be between 0 and 2");
  s->omegaF = wf;
  s->omegaR = wr;
  s->reverse = reverse != 0;
}

void release_trans_plan(const Precond* p) {
  auto* ilu = dynamic_cast<const ILUPrecond*>(p);
  if (ilu) g_trans.erase(ilu);
}

}  // namespace rsg

extern "C" int32_t rsg_sweep_mode(void) { return rsg::g_ring_used.load() ? 2 : rsg::g_cluster_ok.load(); }

// Builds the ring schedule of one ILU(0) sweep of a pattern on the host and
// checks it (rsg::check_ring).  Needs no GPU.
extern "C" rsg_status rsg_sweep_plan_check(int32_t n, const int32_t* row_ptr, const int32_t* col, int32_t sweep,
                                           int32_t ctas, int64_t* stats, char* msg, int32_t msg_len) {
  auto say = [&](const std::string& m) {
    if (msg && msg_len > 0) {
      std::strncpy(msg, m.c_str(), (size_t)msg_len - 1);
      msg[msg_len - 1] = 0;
    }
  };
  if (n <= 0 || !row_ptr || !col || (sweep != 0 && sweep != 1) || (ctas != 8 && ctas != 16)) return RSG_BAD_ARG;
  try {
    std::vector<int> rp(row_ptr, row_ptr + n + 1);
    if (rp[0] != 0) return RSG_BAD_ARG;
    for (int i = 0; i < n; ++i)
      if (rp[i + 1] < rp[i]) return RSG_BAD_ARG;
    std::vector<int> cl(col, col + rp[n]), dg(n, -1);
    for (int i = 0; i < n; ++i)
      for (int q = rp[i]; q < rp[i + 1]; ++q) {
        if (cl[q] < 0 || cl[q] >= n || (q > rp[i] && cl[q] <= cl[q - 1])) return RSG_BAD_ARG;
        if (cl[q] == i) dg[i] = q;
      }
    for (int i = 0; i < n; ++i)
      if (dg[i] < 0) return RSG_MISSING_DIAGONAL;
    rsg::HostRing H;
    if (!rsg::plan_ring(n, rp, cl, dg, sweep == 1, sweep, ctas, rsg::RING_SMEM_MAX, H)) {
      say("no ring schedule");
      return RSG_UNSUPPORTED;
    }
    const std::string err = rsg::check_ring(n, rp, cl, dg, sweep, H);
    say(err);
    if (stats) {
      int64_t pushed = 0, nb = 0;
      for (int v : H.expect) pushed += v;
      for (unsigned short m : H.nbr) nb = std::max<int64_t>(nb, __builtin_popcount(m));
      stats[0] = H.nlev;
      stats[1] = H.R;
      stats[2] = pushed;
      stats[3] = nb;
    }
    return err.empty() ? RSG_OK : RSG_OUT_OF_PATTERN;
  } catch (const std::exception& e) {
    say(e.what());
    return RSG_CUDA_ERROR;
  }
}
