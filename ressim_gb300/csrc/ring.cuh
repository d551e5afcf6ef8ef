// Level walk of an ILU(0) triangular sweep on one thread-block cluster,
// values exchanged through distributed shared memory (used by precond.cu's
// k_sweep_ring and by the ensemble solver in ensemble.cu).  Rows are summed
// in CSR order, as UnitLowerCompRowMatrix.solve / UpperCompRowMatrix.solve
// (mtj/src/no/uib/cipr/matrix/sparse/ILU.java:54-140) do, so the results
// equal the sequential loops bit for bit.
#pragma once
#include <cooperative_groups.h>

#include "linalg.cuh"

namespace rsg {

namespace cg = cooperative_groups;

enum SweepKind { SW_ILU_LOWER = 0, SW_ILU_UPPER = 1, SW_SSOR_FWD = 2, SW_SSOR_BWD = 3, SW_ILU_LOWER_T = 4 };

// ILU sweeps on one thread-block cluster whose CTAs own contiguous blocks
// of rows, with the computed values exchanged through distributed shared
// memory.  A row-block partition keeps most of a row's operands inside its
// CTA: on a stencil pattern in natural order a block of grid planes reads
// only the edge plane of the block before it (lower sweep) or after it
// (upper sweep), so each value is pushed to the few CTAs that read it
// instead of to every CTA.
//
// Layout (RingPlan): every plan level has RING_SLICES slices; CTA c owns
// slices [c W, c W + W) of each level (W = RING_SLICES / C warps, one slice
// per warp), holding its rows of that level packed from the first slot.  A
// level of the dependency schedule whose rows of one CTA exceed W * 32 is
// split into consecutive plan levels (rows of one level are independent, so
// any order among them is valid).
//
// Every CTA keeps a replica of the last R levels (a ring of R level slots of
// RING_SLICES * 32 values in its shared memory; each value at its slot
// position in the level).  The lane that computes a row writes the value into
// its own replica; the even lane of each lane pair pushes the pair's two
// values with st.async into the replicas of the CTAs that read either of
// them (a per-pair CTA mask from the plan).  Completion is counted in bytes on
// the receiving CTA's mbarrier of that level slot, armed with expect_tx from
// the plan's table of values each CTA receives per level.  Besides data, each
// CTA pushes one 8-byte token per level to each CTA it exchanges values with
// (its neighbours: the mask is symmetric) when it starts level l, meaning
// "finished level l-1"; the token counts towards the neighbour's slot of
// level l + S (S = the plan's slack), so a CTA starts level l only after
// every neighbour has finished level l-2-S.  Data flows one way between two
// CTAs (a lower sweep's blocks read earlier blocks), so with S > 0 each CTA
// can run up to S + 1 levels ahead of the CTA it feeds: the pushes of level
// l-1 have landed long before the reader starts level l, and the transfer
// latency leaves the chain of levels.
//
// Slot reuse (R >= lookback + 2 + S and R >= 2 S + 2): a CTA pushing level l
// into a neighbour's slot l mod R has seen that neighbour's token for level
// l-2-S (in its own wait for level l-1), so the neighbour computes level
// l-1-S or later, whose operands lie in levels >= l-1-S-lookback > l-R; slot
// l mod R held level l-R, which it no longer reads, and that slot's mbarrier
// phase for level l-R has completed (the neighbour waited on it at level
// l-R+1 <= l-1-S).  A token for level l+S lands in slot (l+S) mod R, whose
// phase for level l+S-R completed at level l+S-R+1 <= l-1-S.  Bytes of a
// level can reach a slot before its owner arms it for that level: the phase
// cannot complete before the owner's own arrival.
struct RingArgs {
  int nlev, R;
  int slack;                   // levels a CTA may run ahead of a neighbour beyond one
  const int* slice_base;       // per slice: offset of its first entry
  const int* row;              // per slot: row id, -1 if empty
  const int* len;              // per slot: entries of the row
  const int* ridx;             // per entry: ring index of the column's value
  const unsigned short* pmask; // per slot (even lanes): CTAs that read either value of the pair
  const int* expect;           // per level and CTA: values pushed to it
  const unsigned short* nbr;   // per CTA: CTAs it exchanges values or tokens with
  int* err;                    // set to 1 + level when a wait runs out
};

template <typename T>
struct RingVals {
  const T* val;
  const T* diag;
  const T* b;
  T* x;
  const int* active;
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

__device__ __forceinline__ void mbar_inval(unsigned a) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
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

constexpr int RING_TOKEN_BYTES = 8;
constexpr int RING_MAX_CTAS = 16;
constexpr int RING_SLOT = RING_SLICES * 32;  // values per level slot
constexpr size_t RING_SMEM_MAX = 200 * 1024;

// Dynamic shared memory of k_sweep_ring: ring, mbarriers, tokens.
template <typename T>
__host__ __device__ inline size_t ring_smem_bytes(int R) {
  return sizeof(T) * (size_t)R * RING_SLOT + 8 * (size_t)R + RING_TOKEN_BYTES * (size_t)RING_MAX_CTAS;
}

struct RingMeta {
  int row, len, base, slot;
  unsigned pm;
};

template <typename T, int MAXW>
struct RingRow {
  int row, len, base;
  unsigned pm;
  T b, d;
  T v[MAXW];
  int c[MAXW];
};

__device__ __forceinline__ RingMeta ring_meta(const RingArgs& g, int l, int gwarp, int lane) {
  RingMeta m{-1, 0, 0, 0, 0u};
  if (l >= g.nlev) return m;
  const int s = l * RING_SLICES + gwarp;
  m.slot = s * 32 + lane;
  m.row = g.row[m.slot];
  m.len = g.len[m.slot];
  m.base = g.slice_base[s] + lane;
  m.pm = g.pmask[m.slot];
  return m;
}

template <int KIND, typename T, int MAXW>
__device__ __forceinline__ void ring_coeffs(const RingArgs& g, const RingVals<T>& a, const RingMeta& m,
                                            RingRow<T, MAXW>& p) {
  p.row = m.row;
  p.len = m.row >= 0 ? m.len : 0;
  p.base = m.base;
  p.pm = m.row >= 0 ? m.pm : 0u;
  p.b = __ldcg(a.b + (m.row >= 0 ? m.row : 0));  // b may come from other SMs of the same launch
  if (KIND == SW_ILU_UPPER) p.d = a.diag[m.row >= 0 ? m.slot : 0];
#pragma unroll
  for (int k = 0; k < MAXW; ++k)
    if (k < p.len) {
      p.v[k] = a.val[p.base + 32 * k];
      p.c[k] = g.ridx[p.base + 32 * k];
    }
}

// OR of pred over the first NT threads of the CTA (named barrier ID; the
// other threads do not take part).
template <int ID, int NT>
__device__ __forceinline__ int bar_red_or(int pred) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.s32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\t"
      "selp.s32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"(pred), "n"(ID), "n"(NT)
      : "memory");
  return r;
}

// One term of a row's sum: sum + v x, rounded after the product and after
// the sum (MTJ's arithmetic) or, for FP64 with FMA, once (a fused
// multiply-add: half the FP64 instructions of a level, which set about half
// its cost).  FP32 walks always round twice: their arithmetic is cheap, and
// fusing them made the mixed-precision step 9% slower.
template <bool FMA, typename T>
__device__ __forceinline__ T row_term(T sum, T v, T x) {
  if constexpr (FMA && sizeof(T) == 8) return __fma_rn(v, x, sum);
  else return sum + v * x;
}

// The level loop of ring_walk, run by the walking warps only (the first
// RING_SLICES / RING_CTAS warps of each CTA; their barrier is the CTA barrier
// when they are the whole CTA, else named barrier 1).  Ends when everything
// owed to this CTA has landed; false when a wait ran out (g.err is set).
template <int KIND, typename T, int MAXW, int RING_CTAS, int CTA_THREADS, bool FMA>
__device__ __forceinline__ bool ring_levels(const RingArgs& g, const RingVals<T>& a, T* ring, unsigned ring0,
                                            unsigned bar0, unsigned tok0, unsigned rank) {
  constexpr int RING_WARPS = RING_SLICES / RING_CTAS;
  constexpr int WALK_THREADS = RING_WARPS * 32;
  const int lane = threadIdx.x & 31;
  const int gwarp = (int)rank * RING_WARPS + (threadIdx.x >> 5);
  bool ok = true;
  const unsigned nbr = g.nbr[rank];
  const unsigned token_tx = RING_TOKEN_BYTES * __popc(nbr);
  RingRow<T, MAXW> cur, nxt;
  RingMeta m1 = ring_meta(g, 1, gwarp, lane);
  {
    const RingMeta m0 = ring_meta(g, 0, gwarp, lane);
    ring_coeffs<KIND, T, MAXW>(g, a, m0, cur);
  }
  int exp_cur = (threadIdx.x == 0 && g.nlev > 0) ? g.expect[rank] : 0;
  int slot_l = 0, par_l = 0, slot_p = 0, par_p = 0;  // level l and level l-1
  for (int l = 0; l < g.nlev; ++l) {
    if (threadIdx.x == 0) mbar_arm(bar0 + 8 * slot_l, (unsigned)(exp_cur * sizeof(T)) + (l >= g.slack ? token_tx : 0u));
    const int exp_nxt = (threadIdx.x == 0 && l + 1 < g.nlev) ? g.expect[(l + 1) * RING_CTAS + rank] : 0;
    const RingMeta m2 = ring_meta(g, l + 2, gwarp, lane);
    ring_coeffs<KIND, T, MAXW>(g, a, m1, nxt);
    // one thread waits for the level's values and tokens; the barrier below
    // releases the others (fewer instructions in flight than every thread
    // polling the mbarrier)
    const int late = (l > 0 && threadIdx.x == 0) ? !mbar_wait(bar0 + 8 * slot_p, par_p) : 0;
    int any_late;
    if constexpr (CTA_THREADS == WALK_THREADS) any_late = __syncthreads_or(late);
    else any_late = bar_red_or<1, WALK_THREADS>(late);
    if (any_late) {
      if (threadIdx.x == 0) atomicCAS(g.err, 0, 1 + l);
      ok = false;
      break;
    }
    if (threadIdx.x == 0 && l + g.slack < g.nlev) {
      // this CTA has finished level l-1: a token for the neighbours' slot of level l + slack
      const int ts = slot_l + g.slack < g.R ? slot_l + g.slack : slot_l + g.slack - g.R;
      for (unsigned m = nbr; m; m &= m - 1) {
        const unsigned c = __ffs(m) - 1;
        push_b64(cluster_addr(tok0, c) + RING_TOKEN_BYTES * rank, (unsigned long long)l,
                 cluster_addr(bar0, c) + 8 * ts);
      }
    }
    const bool act = cur.row >= 0;
    T v = 0;
    const int own = slot_l * RING_SLOT + gwarp * 32 + lane;
    if (act) {
      T sum = 0;
#pragma unroll
      for (int k = 0; k < MAXW; ++k)
        if (k < cur.len) sum = row_term<FMA>(sum, cur.v[k], ring[cur.c[k]]);
      for (int k = MAXW; k < cur.len; ++k) {
        const int q = cur.base + 32 * k;
        sum = row_term<FMA>(sum, a.val[q], ring[g.ridx[q]]);
      }
      v = (KIND == SW_ILU_LOWER) ? cur.b - sum : (cur.b - sum) / cur.d;
      ring[own] = v;
      a.x[cur.row] = v;
    }
    // the even lane of each pair pushes both values to the CTAs that read
    // them (rows of a level are packed from the CTA's first slot, so a pair
    // with an active odd lane has an active even lane; an unused odd slot is
    // never read)
    const T v_odd = __shfl_down_sync(0xffffffffu, v, 1);
    if (act && !(lane & 1)) {
      const unsigned off = (unsigned)(own * sizeof(T)), boff = (unsigned)(8 * slot_l);
      for (unsigned m = cur.pm; m; m &= m - 1) {
        const unsigned c = __ffs(m) - 1;
        push_pair(cluster_addr(ring0, c) + off, v, v_odd, cluster_addr(bar0, c) + boff);
      }
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
  if (ok && g.nlev > 0) {
    // everything owed to this CTA lands before any CTA may exit
    if (!mbar_wait(bar0 + 8 * slot_p, par_p)) {
      atomicCAS(g.err, 0, 1 + g.nlev);
      ok = false;
    }
  }
  return ok;
}

// One walk of the levels by the calling cluster (all its threads call it,
// with blockDim.x == CTA_THREADS).  The first RING_SLICES / RING_CTAS warps
// of each CTA walk; further warps (a persistent kernel that wants more warps
// for its other phases) only take part in the cluster barriers at the start
// and the end.  smem: the dynamic shared memory, at least
// ring_smem_bytes<T>(g.R).  Returns false when a wait ran out (g.err is
// set); the caller must then stop using the cluster's shared memory for
// walks.  On success every mbarrier is invalidated again, so the same memory
// can hold the next walk.  FMA: an FP64 row's terms as fused multiply-adds
// instead of MTJ's product-then-sum rounding.
template <int KIND, typename T, int MAXW, int RING_CTAS, int CTA_THREADS = RING_SLICES / RING_CTAS * 32,
          bool FMA = false>
__device__ __forceinline__ bool ring_walk(const RingArgs& g, const RingVals<T>& a, unsigned char* smem) {
  constexpr int RING_WARPS = RING_SLICES / RING_CTAS;
  constexpr int WALK_THREADS = RING_WARPS * 32;
  static_assert(CTA_THREADS >= WALK_THREADS && CTA_THREADS % 32 == 0, "the walk needs its warps");
  T* ring = reinterpret_cast<T*>(smem);
  unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem + sizeof(T) * (size_t)g.R * RING_SLOT);
  unsigned long long* tok = bar + g.R;
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const unsigned ring0 = smem_addr(ring), bar0 = smem_addr(bar), tok0 = smem_addr(tok);
  if (threadIdx.x < g.R) mbar_init(bar0 + 8 * threadIdx.x, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  cluster.sync();  // every replica's barriers exist before the first push
  bool ok = true;
  if (CTA_THREADS == WALK_THREADS || threadIdx.x < WALK_THREADS)
    ok = ring_levels<KIND, T, MAXW, RING_CTAS, CTA_THREADS, FMA>(g, a, ring, ring0, bar0, tok0, rank);
  cluster.sync();
  if (*(volatile int*)g.err != 0) {
    // a wait ran out somewhere: give pushes still in flight time to land
    for (int i = 0; i < 64; ++i) __nanosleep(1000);
    return false;
  }
  // every phase has completed and nothing is in flight (each CTA waited for
  // all it was owed before the barrier above)
  if (threadIdx.x < g.R) mbar_inval(bar0 + 8 * threadIdx.x);
  __syncthreads();
  return ok;
}

template <int KIND, typename T, int MAXW, int RING_CTAS, bool FMA>
__global__ void __launch_bounds__(RING_SLICES / RING_CTAS * 32) k_sweep_ring(RingArgs g, RingVals<T> a) {
  if (a.active && *a.active != 0) return;  // uniform over the cluster
  extern __shared__ __align__(16) unsigned char smem[];
  ring_walk<KIND, T, MAXW, RING_CTAS, RING_SLICES / RING_CTAS * 32, FMA>(g, a, smem);
}


}  // namespace rsg
