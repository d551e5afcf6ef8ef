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

#include "linalg.cuh"

namespace cg = cooperative_groups;

namespace rsg {

enum SweepKind { SW_ILU_LOWER = 0, SW_ILU_UPPER = 1, SW_SSOR_FWD = 2, SW_SSOR_BWD = 3, SW_ILU_LOWER_T = 4 };

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

// ILU sweeps with the computed values exchanged through distributed shared
// memory instead of L2.  Every CTA of the cluster keeps a replica of the
// values of the last R levels (a ring of R level slots in its shared
// memory).  The lane that computes a row writes the value into its own
// replica and pushes it into the other CTAs' replicas with st.async, whose
// completion is counted in bytes on the receiving CTA's mbarrier of that
// level slot.  Besides its rows, each CTA pushes one 8-byte token per level
// to every other CTA once it has finished the previous level, so a level's
// phase completes only when every CTA is done with the level before it: no
// CTA runs more than one level ahead of another.  A CTA starts level l once
// its mbarrier of level l-1 has seen every byte owed to it (armed with
// expect_tx from a host-built table) and a CTA barrier has published its
// own rows; all operand gathers are then local shared-memory loads and there
// is no cluster-wide barrier per level.
//
// Slot reuse: a CTA pushing level l into slot l mod R has seen the token of
// every CTA for level l-1, so each of them has finished level l-2 and is at
// most computing level l-1, whose operands lie in levels >= l-1-(R-2) when
// R >= lookback + 2; slot l mod R held level l-R, which nobody reads any
// more, and its mbarrier phase for level l-R has completed.
struct RingArgs {
  int R;                // ring depth in levels (>= lookback + 2)
  int slot;             // values per level slot (slices x 32)
  const int* ridx;      // per entry slot: ring index of the column's value
  const int* expect;    // per level and CTA rank: rows pushed by the other CTAs
  int* err;             // set to 1 + level when a wait runs out
};

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned cluster_addr(unsigned a, unsigned rank) {
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__device__ __forceinline__ void mbar_init(unsigned a, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arm(unsigned a, unsigned tx) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(tx) : "memory");
}

__device__ __forceinline__ bool mbar_test(unsigned a, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false when the phase did not complete within the limit
__device__ __forceinline__ bool mbar_wait(unsigned a, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i)
    if (mbar_test(a, parity)) return true;
  return false;
}

__device__ __forceinline__ void push_b64(unsigned remote, unsigned long long v, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(remote), "l"(v),
               "r"(rbar)
               : "memory");
}

// two neighbouring values (16 or 8 bytes) in one push: the even lane of a
// lane pair sends its own and its odd neighbour's value, which halves the
// number of transfers each receiving mbarrier counts
__device__ __forceinline__ void push_pair(unsigned remote, double v0, double v1, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];" ::"r"(remote),
               "l"((unsigned long long)__double_as_longlong(v0)), "l"((unsigned long long)__double_as_longlong(v1)),
               "r"(rbar)
               : "memory");
}

__device__ __forceinline__ void push_pair(unsigned remote, float v0, float v1, unsigned rbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];" ::"r"(remote),
               "r"(__float_as_uint(v0)), "r"(__float_as_uint(v1)), "r"(rbar)
               : "memory");
}

template <int KIND, typename T, int MAXW>
__device__ __forceinline__ void load_ring_coeffs(const SweepArgs<T>& a, const RingArgs& g, const int* ls,
                                                 const SlotMeta& m, int l, int gwarp, int lane,
                                                 RowPrefetch<T, MAXW>& p) {
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
      p.c[k] = g.ridx[p.base + 32 * k];
    }
}

constexpr int RING_TOKEN_BYTES = 8;
constexpr int RING_MAX_CTAS = 16;

// Dynamic shared memory of k_sweep_ring: ring, mbarriers, tokens, level offsets.
template <typename T>
__host__ __device__ inline size_t ring_smem_bytes(int R, int slot, int nlev) {
  return sizeof(T) * (size_t)R * slot + 8 * (size_t)R + RING_TOKEN_BYTES * (size_t)RING_MAX_CTAS +
         4 * (size_t)(nlev + 1);
}

template <int KIND, typename T, int MAXW, int RING_CTAS>
__global__ void __launch_bounds__(RING_SLICES / RING_CTAS * 32) k_sweep_ring(SweepArgs<T> a, RingArgs g) {
  constexpr int RING_WARPS = RING_SLICES / RING_CTAS;
  if (a.active && *a.active != 0) return;  // uniform over the cluster
  extern __shared__ __align__(16) unsigned char smem[];
  T* ring = reinterpret_cast<T*>(smem);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + sizeof(T) * (size_t)g.R * g.slot);
  unsigned long long* tok = bar + g.R;
  int* ls = reinterpret_cast<int*>(tok + RING_MAX_CTAS);
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)rank * RING_WARPS + (threadIdx.x >> 5);
  const unsigned ring0 = smem_addr(ring), bar0 = smem_addr(bar), tok0 = smem_addr(tok);
  if (threadIdx.x < g.R) mbar_init(bar0 + 8 * threadIdx.x, 1);
  for (int q = threadIdx.x; q <= a.nlev; q += blockDim.x) ls[q] = a.level_slices[q];
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  cluster.sync();  // every replica's barriers exist before the first push
  unsigned rring[RING_CTAS], rbar[RING_CTAS];
#pragma unroll
  for (int c = 0; c < RING_CTAS; ++c) {
    rring[c] = cluster_addr(ring0, c);
    rbar[c] = cluster_addr(bar0, c);
  }
  RowPrefetch<T, MAXW> cur, nxt;
  SlotMeta m1 = load_meta(a, ls, 1, gwarp, lane);
  {
    SlotMeta m0 = load_meta(a, ls, 0, gwarp, lane);
    load_ring_coeffs<KIND, T, MAXW>(a, g, ls, m0, 0, gwarp, lane, cur);
  }
  const unsigned token_tx = RING_TOKEN_BYTES * (RING_CTAS - 1);
  int exp_cur = (threadIdx.x == 0 && a.nlev > 0) ? g.expect[rank] : 0;
  int slot_l = 0, par_l = 0, slot_p = 0, par_p = 0;  // level l and level l-1
  bool ok = true;
  for (int l = 0; l < a.nlev; ++l) {
    if (threadIdx.x == 0) mbar_arm(bar0 + 8 * slot_l, (unsigned)(exp_cur * sizeof(T)) + token_tx);
    const int exp_nxt = (threadIdx.x == 0 && l + 1 < a.nlev) ? g.expect[(l + 1) * RING_CTAS + rank] : 0;
    const SlotMeta m2 = load_meta(a, ls, l + 2, gwarp, lane);
    load_ring_coeffs<KIND, T, MAXW>(a, g, ls, m1, l + 1, gwarp, lane, nxt);
    const int late = (l > 0) ? !mbar_wait(bar0 + 8 * slot_p, par_p) : 0;
    if (__syncthreads_or(late)) {
      if (threadIdx.x == 0) atomicCAS(g.err, 0, 1 + l);
      ok = false;
      break;
    }
    if (threadIdx.x == 0) {
      // this CTA has finished level l-1
#pragma unroll
      for (int c = 0; c < RING_CTAS; ++c)
        if (c != (int)rank)
          push_b64(cluster_addr(tok0, c) + RING_TOKEN_BYTES * rank, (unsigned long long)l, rbar[c] + 8 * slot_l);
    }
    const bool act = cur.row >= 0;
    T v = 0;
    const int own = slot_l * g.slot + gwarp * 32 + lane;
    if (act) {
      T sum = 0;
#pragma unroll
      for (int k = 0; k < MAXW; ++k)
        if (k < cur.len) sum += cur.v[k] * ring[cur.c[k]];
      for (int k = MAXW; k < cur.len; ++k) {
        const int q = cur.base + 32 * k;
        sum += a.val[q] * ring[g.ridx[q]];
      }
      v = (KIND == SW_ILU_LOWER) ? cur.b - sum : (cur.b - sum) / cur.d;
      ring[own] = v;
      a.x[cur.row] = v;
    }
    // the even lane of each pair pushes both values (rows of a level are
    // packed from its first slot, so a pair with an active odd lane has an
    // active even lane; an unused odd slot is never read)
    const T v_odd = __shfl_down_sync(0xffffffffu, v, 1);
    if (act && !(lane & 1)) {
      const unsigned off = (unsigned)(own * sizeof(T)), boff = (unsigned)(8 * slot_l);
#pragma unroll
      for (int c = 0; c < RING_CTAS; ++c)
        if (c != (int)rank) push_pair(rring[c] + off, v, v_odd, rbar[c] + boff);
    }
    cur = nxt;
    m1 = m2;
    exp_cur = exp_nxt;
    slot_p = slot_l;
    par_p = par_l;
    if (++slot_l == g.R) {
      slot_l = 0;
      par_l ^= 1;
    }
  }
  if (ok && a.nlev > 0) {
    // everything owed to this CTA lands before any CTA may exit
    if (!mbar_wait(bar0 + 8 * slot_p, par_p)) {
      atomicCAS(g.err, 0, 1 + a.nlev);
      ok = false;
    }
  }
  cluster.sync();
  if (*(volatile int*)g.err != 0) {
    // a wait ran out somewhere: give pushes still in flight time to land
    for (int i = 0; i < 64; ++i) __nanosleep(1000);
  }
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
  // push-ring schedule (lower or upper ILU parts only)
  std::vector<int> ridx, expect[2];
  P.ring_R = 0;
  if (entries != 2) {
    int max_sl = 0, look = 0;
    for (int l = 0; l < nlev; ++l) max_sl = std::max(max_sl, level_slices[l + 1] - level_slices[l]);
    std::vector<int> ring_pos(n);  // slice offset within the level * 32 + lane
    for (int l = 0; l < nlev; ++l)
      for (int t = 0; t < cnt[l + 1] - cnt[l]; ++t) ring_pos[order[cnt[l] + t]] = t;
    for (int i = 0; i < n; ++i) {
      int b0, b1, c0, c1;
      row_entries(i, b0, b1, c0, c1);
      for (int q = b0; q < b1; ++q) look = std::max(look, lev[i] - lev[cl[q]]);
    }
    const int R = look + 2;
    if (max_sl <= RING_SLICES && R <= 32) {
      P.ring_R = R;
      P.ring_slot = max_sl * 32;
      ridx.assign(col.size(), 0);
      for (int s = 0; s < ns; ++s)
        for (int lane = 0; lane < 32; ++lane) {
          int r = row[(size_t)s * 32 + lane];
          if (r < 0) continue;
          for (int k = 0; k < len[(size_t)s * 32 + lane]; ++k) {
            int c = col[base[s] + 32 * k + lane];
            ridx[base[s] + 32 * k + lane] = (lev[c] % R) * P.ring_slot + ring_pos[c];
          }
        }
      for (int e = 0; e < 2; ++e) {
        const int C = 8 << e, W = RING_SLICES / C;
        auto& ex = expect[e];
        ex.assign((size_t)nlev * C, 0);
        for (int l = 0; l < nlev; ++l) {
          const int rows = cnt[l + 1] - cnt[l];
          // values pushed by each CTA: its rows, rounded up to whole lane pairs
          int total = 0;
          std::vector<int> sent(C);
          for (int c = 0; c < C; ++c) {
            const int own = std::min(std::max(rows - c * W * 32, 0), W * 32);
            sent[c] = 2 * ((own + 1) / 2);
            total += sent[c];
          }
          for (int c = 0; c < C; ++c) ex[(size_t)l * C + c] = total - sent[c];
        }
      }
    }
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
  if (P.ring_R) {
    P.ridx.resize(ridx.size());
    up(P.ridx, ridx);
    for (int e = 0; e < 2; ++e) {
      P.ring_expect[e].resize(expect[e].size());
      up(P.ring_expect[e], expect[e]);
    }
  }
  if (with_diag) {
    P.diag_src.resize(dsrc.size());
    P.diag.resize(dsrc.size());
    P.diagf.resize(dsrc.size());
    up(P.diag_src, dsrc);
  }
  ctx.sync();
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

// Push-ring launch: one cluster with the ring, its mbarriers and the level
// offsets in dynamic shared memory.  FP64 walks use a cluster of 16 CTAs
// (4 warps each) when the device schedules one, since their time per level
// is bound by the SMs' FP64 rate; FP32 walks use 8 CTAs of 8 warps.
// RSG_SWEEP=pipelined switches the ring off, RSG_RING_CTAS=8|16 forces the
// cluster size.  Returns false when the ring does not fit or no cluster can
// be scheduled.
static std::atomic<int> g_ring_mode{-1};  // -1: not read; 0 off; 1 on
static int g_ring_ctas = 0;               // forced cluster size, 0: automatic
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

constexpr size_t RING_SMEM_MAX = 200 * 1024;

template <int KIND, typename T, int CTAS>
static bool launch_ring_n(Context& ctx, const char* name, const SweepPlan& P, const SweepArgs<T>& a, size_t smem) {
  auto kern = k_sweep_ring<KIND, T, 16, CTAS>;
  static std::atomic<int> ok{0};  // per instantiation: 0 not probed, 1 schedulable, -1 not
  if (!ok) {
    std::lock_guard<std::mutex> lk(g_probe_mu);
    if (!ok) ok = ring_schedulable(kern, CTAS, RING_SMEM_MAX) ? 1 : -1;
  }
  if (ok < 0) return false;
  RingArgs g{P.ring_R, P.ring_slot, P.ridx.get(), P.ring_expect[CTAS == 16].get(), ctx.dev_err.get()};
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
  RSG_CUDA(cudaLaunchKernelEx(&cfg, kern, a, g));
  g_ring_used = true;
  return true;
}

template <int KIND, typename T>
static bool launch_ring(Context& ctx, const char* name, const SweepPlan& P, const SweepArgs<T>& a) {
  if (g_ring_mode < 0) {
    std::lock_guard<std::mutex> lk(g_probe_mu);
    if (g_ring_mode < 0) {
      const char* c = getenv("RSG_RING_CTAS");
      g_ring_ctas = c ? atoi(c) : 0;
      const char* e = getenv("RSG_SWEEP");
      g_ring_mode = (e && std::string(e) == "pipelined") ? 0 : 1;
    }
  }
  if (!g_ring_mode || !P.ring_R) return false;
  const size_t smem = ring_smem_bytes<T>(P.ring_R, P.ring_slot, P.nlev);
  if (smem > RING_SMEM_MAX) return false;
  const bool want16 = g_ring_ctas ? g_ring_ctas == 16 : sizeof(T) == 8;
  if (want16 && launch_ring_n<KIND, T, 16>(ctx, name, P, a, smem)) return true;
  return launch_ring_n<KIND, T, 8>(ctx, name, P, a, smem);
}

template <int KIND, typename T>
static void run_sweep(Context& ctx, const char* name, const SweepPlan& P, const T* val, const T* diag, const T* b,
                      T* x, T* xx, T omega, const int* active) {
  SweepArgs<T> a{P.nlev, P.level_slices.get(), P.slice_base.get(), P.row.get(), P.len.get(), P.col.get(), val, diag,
                 b, x, xx, omega, active};
  if constexpr (KIND == SW_ILU_LOWER || KIND == SW_ILU_UPPER)
    if (launch_ring<KIND, T>(ctx, name, P, a)) return;
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
  }

  void apply(const double* b, double* x, const int* active) override {
    // L.solve(b, y); U.solve(y, x)
    run_sweep<SW_ILU_LOWER, double>(*ctx, "ilu_lower", Lp, Lp.val.get(), nullptr, b, y.get(), nullptr, 0.0, active);
    run_sweep<SW_ILU_UPPER, double>(*ctx, "ilu_upper", Up, Up.val.get(), Up.diag.get(), y.get(), x, nullptr, 0.0,
                                    active);
  }
  void apply_f32(const float* b, float* x, const int* active) override {
    run_sweep<SW_ILU_LOWER, float>(*ctx, "ilu_lower_f32", Lp, Lp.valf.get(), nullptr, b, yf.get(), nullptr, 0.0f,
                                   active);
    run_sweep<SW_ILU_UPPER, float>(*ctx, "ilu_upper_f32", Up, Up.valf.get(), Up.diagf.get(), yf.get(), x, nullptr,
                                   0.0f, active);
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
      A = &M;
      pattern_id = M.rowptr.get();
    }
    plan_values(*ctx, Fp, M.val.get(), true, false);
    plan_values(*ctx, Bp, M.val.get(), true, false);
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
