// Smoothed-aggregation AMG preconditioner (mtj/src/no/uib/cipr/matrix/
// sparse/AMG.java) with the parameters of AMG() (:204-206): SSOR(1, 1.85)
// pre-smoothing and SSOR(1.85, 1) post-smoothing (reverse sweeps), one each,
// a V-cycle, coarsening until at most 40 rows, Jacobi-smoothed prolongation
// with omega 2/3, and a dense LU of the coarsest operator.
//
// The whole setup runs on the GPU:
//  * strength of connection and the initial free set, one thread per row;
//  * createInitialAggregates and createFinalAggregates are greedy scans in
//    node order whose outcome depends on every earlier decision, so one CTA
//    walks the nodes with the free set as a bitmap in shared memory;
//  * enlargeAggregates only reads the aggregates of the first phase, so it
//    runs one thread per node;
//  * the smoothed prolongation, A*P and P'*(A*P) run one warp per output
//    row.  Each lane owns the output columns congruent to its lane id and
//    walks all terms of the row in the reference's order, so every output
//    value is summed in exactly the order of the Java loops.
// The V-cycle reuses the level-scheduled SSOR sweeps of precond.cu.
//
// Equivalent-form restatements (also in the oracle): the Galerkin product
// sums only non-zero terms (createGalerkinSlow forms dense columns; skipped
// terms are exact zeros), and enlargeAggregates breaks ties between equally
// overlapping aggregates in ascending node order (MTJ's order is that of a
// java.util.HashSet).
#include <algorithm>
#include <mutex>
#include <cmath>
#include <string>

#include "linalg.cuh"

namespace rsg {

void set_ssor_params(Precond* p, double wf, double wr, int reverse);

namespace {

constexpr int AMG_MIN = 40;              // AMG() min
constexpr double AMG_OMEGA = 2.0 / 3.0;  // AMG() omega
constexpr int LANE_SLOTS = 16;           // accumulator slots per lane (512 per row)
constexpr int AMG_WARPS = 4;             // warps per block of the row kernels
constexpr int PHASE_CHUNK = 512;         // rows staged per step of the greedy scans
constexpr int PHASE_ENTRIES = 12288;     // entries staged per step
constexpr int COARSE_MAX = 512;          // largest coarsest operator factorised densely

enum AmgFlag { AF_OK = 0, AF_SLOTS = 1, AF_CHUNK = 2 };

// ------------------------------------------------------------- strength ----
// findNodeNeighborhood (AMG.java:470-494) and createInitialR (:500-518)
__global__ void k_strength(int n, const int* __restrict__ rp, const int* __restrict__ col,
                           const double* __restrict__ val, const int* __restrict__ diag, double eps,
                           unsigned char* __restrict__ S, unsigned char* __restrict__ R0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double aii = val[diag[i]];
  bool off = false;
  for (int q = rp[i]; q < rp[i + 1]; ++q) {
    const int j = col[q];
    const double aij = val[q];
    const double ajj = val[diag[j]];
    S[q] = fabs(aij) >= eps * sqrt(aii * ajj);
    if (!off && j != i && aij != 0) off = true;
  }
  R0[i] = off;
}

// ------------------------------------------------------ greedy phases ----
// One CTA walks the nodes in order.  Rows are staged a chunk at a time into
// shared memory by the whole CTA; warp 0 then decides node by node with the
// free set held as a bitmap (bit set = free).
struct PhaseArgs {
  int n;
  const int* rp;
  const int* col;
  const unsigned char* S;
  const unsigned char* free0;  // free set at entry (1 byte per node)
  const int* prev;             // phase 1: nullptr; phase 3: assigned aggregate so far
  int* agg;                    // out: aggregate formed in this phase (-1: none)
  int* count;                  // in: first id; out: next id
  unsigned* gbits;             // bitmap in global memory when it does not fit in shared memory
  int* flag;
  int final_phase;             // 0: createInitialAggregates, 1: createFinalAggregates
};

__global__ void __launch_bounds__(1024) k_agg_greedy(PhaseArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  int* srp = reinterpret_cast<int*>(sm);                 // PHASE_CHUNK + 1
  int* scol = srp + PHASE_CHUNK + 1;                     // PHASE_ENTRIES
  unsigned char* sS = reinterpret_cast<unsigned char*>(scol + PHASE_ENTRIES);  // PHASE_ENTRIES
  unsigned* bits = a.gbits ? a.gbits : reinterpret_cast<unsigned*>(sS + PHASE_ENTRIES);
  volatile unsigned* vbits = bits;  // read back after other lanes' atomics
  const int nw = (a.n + 31) / 32;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) {
    unsigned b = 0;
    for (int t = 0; t < 32; ++t) {
      const int i = w * 32 + t;
      if (i < a.n && a.free0[i]) b |= 1u << t;
    }
    bits[w] = b;
  }
  for (int i = threadIdx.x; i < a.n; i += blockDim.x) a.agg[i] = -1;
  __syncthreads();
  int next = *a.count;
  const int lane = threadIdx.x & 31;
  for (int r0 = 0; r0 < a.n; r0 += PHASE_CHUNK) {
    const int rows = min(PHASE_CHUNK, a.n - r0);
    const int e0 = a.rp[r0], e1 = a.rp[r0 + rows];
    const bool staged = (e1 - e0) <= PHASE_ENTRIES;
    for (int t = threadIdx.x; t <= rows; t += blockDim.x) srp[t] = a.rp[r0 + t] - e0;
    if (staged)
      for (int q = threadIdx.x; q < e1 - e0; q += blockDim.x) {
        scol[q] = a.col[e0 + q];
        sS[q] = a.S[e0 + q];
      }
    __syncthreads();
    if (threadIdx.x < 32) {
      for (int t = 0; t < rows; ++t) {
        const int i = r0 + t;
        const bool ifree = (vbits[i >> 5] >> (i & 31)) & 1u;  // R[i]
        if (!ifree) continue;
        const int q0 = srp[t], q1 = srp[t + 1];
        if (!a.final_phase) {
          // free &= R[j] for j in N_i; then N_i becomes an aggregate
          bool all = true;
          for (int q = q0 + lane; q < q1; q += 32) {
            const int j = staged ? scol[q] : a.col[e0 + q];
            const bool s = staged ? sS[q] : a.S[e0 + q];
            if (s && !((vbits[j >> 5] >> (j & 31)) & 1u)) all = false;
          }
          all = __all_sync(0xffffffffu, all);
          if (all) {
            for (int q = q0 + lane; q < q1; q += 32) {
              const int j = staged ? scol[q] : a.col[e0 + q];
              const bool s = staged ? sS[q] : a.S[e0 + q];
              if (s) {
                atomicAnd(&bits[j >> 5], ~(1u << (j & 31)));
                a.agg[j] = next;
              }
            }
            next++;
          }
        } else {
          // Cn = {j in N_i : R[j]}, each taken out of the free set
          bool any = false;
          for (int q = q0 + lane; q < q1; q += 32) {
            const int j = staged ? scol[q] : a.col[e0 + q];
            const bool s = staged ? sS[q] : a.S[e0 + q];
            if (s && ((vbits[j >> 5] >> (j & 31)) & 1u)) {
              atomicAnd(&bits[j >> 5], ~(1u << (j & 31)));
              a.agg[j] = next;
              any = true;
            }
          }
          if (__any_sync(0xffffffffu, any)) next++;
        }
        __syncwarp();
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *a.count = next;
}

// enlargeAggregates (AMG.java:554-600): free node i joins the phase-one
// aggregate that first reaches the largest overlap with N_i.
__global__ void k_agg_enlarge(int n, const int* __restrict__ rp, const int* __restrict__ col,
                              const unsigned char* __restrict__ S, const unsigned char* __restrict__ R0,
                              const int* __restrict__ agg1, int* __restrict__ agg2, unsigned char* __restrict__ free2,
                              int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  agg2[i] = -1;
  if (!R0[i] || agg1[i] >= 0) {
    free2[i] = 0;
    return;
  }
  constexpr int K = 32;
  int keys[K], cnt[K];
  int nk = 0, largest = 0, maxValue = 0;
  for (int q = rp[i]; q < rp[i + 1]; ++q) {
    if (!S[q]) continue;
    const int k = agg1[col[q]];
    if (k < 0) continue;
    int s = 0;
    while (s < nk && keys[s] != k) ++s;
    if (s == nk) {
      if (nk == K) {
        atomicCAS(flag, 0, AF_SLOTS);
        return;
      }
      keys[nk] = k;
      cnt[nk++] = 0;
    }
    if (++cnt[s] > maxValue) {
      largest = k;
      maxValue = cnt[s];
    }
  }
  if (maxValue > 0) {
    agg2[i] = largest;
    free2[i] = 0;
  } else {
    free2[i] = 1;
  }
}

__global__ void k_agg_final(int n, const int* __restrict__ a1, const int* __restrict__ a2,
                            const int* __restrict__ a3, int* __restrict__ pt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  pt[i] = a1[i] >= 0 ? a1[i] : (a2[i] >= 0 ? a2[i] : a3[i]);
}

// ---------------------------------------------- lane-owned accumulators ----
// Output column k of a row belongs to lane k % 32; the lane keeps its columns
// in LANE_SLOTS open-addressed slots of shared memory.
struct LaneAcc {
  int* key;
  double* val;
  __device__ void reset() {
    for (int s = 0; s < LANE_SLOTS; ++s) key[s] = -1;
  }
  // returns the slot of k, or -1 when the lane's slots are exhausted
  __device__ int slot(int k) {
    int s = (k >> 5) & (LANE_SLOTS - 1);
    for (int probe = 0; probe < LANE_SLOTS; ++probe) {
      if (key[s] == k) return s;
      if (key[s] == -1) {
        key[s] = k;
        val[s] = 0.0;
        return s;
      }
      s = (s + 1) & (LANE_SLOTS - 1);
    }
    return -1;
  }
};

__device__ __forceinline__ LaneAcc lane_acc(int* skey, double* sval, int warp, int lane) {
  const int off = (warp * 32 + lane) * LANE_SLOTS;
  return LaneAcc{skey + off, sval + off};
}

// Count pass: returns the number of the row's non-zero entries.  Fill pass:
// writes them at out_col/out_val in lane order; k_row_sort then puts each row
// in ascending column order.
__device__ int emit_row(LaneAcc& acc, int lane, int* out_col, double* out_val, bool fill) {
  int mine = 0;
  for (int s = 0; s < LANE_SLOTS; ++s)
    if (acc.key[s] >= 0 && acc.val[s] != 0) mine++;
  int incl = mine;
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (fill) {
    int pos = incl - mine;
    for (int s = 0; s < LANE_SLOTS; ++s)
      if (acc.key[s] >= 0 && acc.val[s] != 0) {
        out_col[pos] = acc.key[s];
        out_val[pos] = acc.val[s];
        pos++;
      }
  }
  return total;
}

__global__ void k_row_sort(int n, const int* __restrict__ rp, int* __restrict__ col, double* __restrict__ val) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int a = rp[i] + 1; a < rp[i + 1]; ++a) {
    const int k = col[a];
    const double v = val[a];
    int b = a - 1;
    while (b >= rp[i] && col[b] > k) {
      col[b + 1] = col[b];
      val[b + 1] = val[b];
      --b;
    }
    col[b + 1] = k;
    val[b + 1] = v;
  }
}

// ----------------------------------------------------------- prolongation ----
// createSmoothedProlongation (AMG.java:810-876), one warp per row of P.
__global__ void __launch_bounds__(AMG_WARPS * 32) k_prolong(int n, const int* __restrict__ rp,
                                                            const int* __restrict__ col,
                                                            const double* __restrict__ val,
                                                            const int* __restrict__ diag,
                                                            const unsigned char* __restrict__ S,
                                                            const int* __restrict__ pt, double omega, int fill,
                                                            int* __restrict__ cnt, const int* __restrict__ optr,
                                                            int* __restrict__ ocol, double* __restrict__ oval,
                                                            int* flag) {
  __shared__ int skey[AMG_WARPS * 32 * LANE_SLOTS];
  __shared__ double sval[AMG_WARPS * 32 * LANE_SLOTS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * AMG_WARPS + warp;
  if (i >= n) return;
  if (pt[i] == -1) {
    if (!fill && lane == 0) cnt[i] = 0;
    return;
  }
  LaneAcc acc = lane_acc(skey, sval, warp, lane);
  acc.reset();
  bool bad = false;
  double weakAij = 0;
  for (int q = rp[i]; q < rp[i + 1]; ++q) {
    const int c = col[q];
    const int k = pt[c];
    if (k == -1) continue;
    const double aij = val[q];
    if (aij != 0 && !S[q]) {
      weakAij += aij;
      continue;
    }
    if ((k & 31) == lane) {
      const int s = acc.slot(k);
      if (s < 0) bad = true;
      else acc.val[s] += aij;
    }
  }
  const int kd = pt[i];
  const double scale = -omega / val[diag[i]];
  if ((kd & 31) == lane) {
    const int s = acc.slot(kd);
    if (s < 0) bad = true;
    else acc.val[s] -= weakAij;
  }
  for (int s = 0; s < LANE_SLOTS; ++s)
    if (acc.key[s] >= 0) acc.val[s] *= scale;
  if ((kd & 31) == lane) {
    const int s = acc.slot(kd);
    if (s >= 0) acc.val[s]++;
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicCAS(flag, 0, AF_SLOTS);
    return;
  }
  __syncwarp();
  const int total = emit_row(acc, lane, fill ? ocol + optr[i] : nullptr, fill ? oval + optr[i] : nullptr, fill);
  if (!fill && lane == 0) cnt[i] = total;
}

// B = A*P, one warp per row of A: B(i,k) = sum over row i of A in CSR order
// of a_ij * P(j,k) (the column products of createGalerkinSlow).
__global__ void __launch_bounds__(AMG_WARPS * 32) k_galerkin_ap(int n, const int* __restrict__ rp,
                                                                const int* __restrict__ col,
                                                                const double* __restrict__ val,
                                                                const int* __restrict__ prp,
                                                                const int* __restrict__ pcol,
                                                                const double* __restrict__ pval, int fill,
                                                                int* __restrict__ cnt, const int* __restrict__ optr,
                                                                int* __restrict__ ocol, double* __restrict__ oval,
                                                                int* flag) {
  __shared__ int skey[AMG_WARPS * 32 * LANE_SLOTS];
  __shared__ double sval[AMG_WARPS * 32 * LANE_SLOTS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * AMG_WARPS + warp;
  if (i >= n) return;
  LaneAcc acc = lane_acc(skey, sval, warp, lane);
  acc.reset();
  bool bad = false;
  for (int q = rp[i]; q < rp[i + 1]; ++q) {
    const double aij = val[q];
    const int j = col[q];
    for (int e = prp[j]; e < prp[j + 1]; ++e) {
      const int k = pcol[e];
      if ((k & 31) != lane) continue;
      const double t = aij * pval[e];
      const int s = acc.slot(k);
      if (s < 0) bad = true;
      else acc.val[s] += t;
    }
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicCAS(flag, 0, AF_SLOTS);
    return;
  }
  __syncwarp();
  const int total = emit_row(acc, lane, fill ? ocol + optr[i] : nullptr, fill ? oval + optr[i] : nullptr, fill);
  if (!fill && lane == 0) cnt[i] = total;
}

// Ac = P'*B, one warp per coarse row k': Ac(k',k) = sum over the rows i of
// column k' of P in ascending order of P(i,k') * B(i,k) (I.transMult).
__global__ void __launch_bounds__(AMG_WARPS * 32) k_galerkin_ptb(int c, const int* __restrict__ qptr,
                                                                 const int* __restrict__ qrow,
                                                                 const double* __restrict__ qval,
                                                                 const int* __restrict__ brp,
                                                                 const int* __restrict__ bcol,
                                                                 const double* __restrict__ bval, int fill,
                                                                 int* __restrict__ cnt, const int* __restrict__ optr,
                                                                 int* __restrict__ ocol, double* __restrict__ oval,
                                                                 int* flag) {
  __shared__ int skey[AMG_WARPS * 32 * LANE_SLOTS];
  __shared__ double sval[AMG_WARPS * 32 * LANE_SLOTS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kp = blockIdx.x * AMG_WARPS + warp;
  if (kp >= c) return;
  LaneAcc acc = lane_acc(skey, sval, warp, lane);
  acc.reset();
  bool bad = false;
  for (int q = qptr[kp]; q < qptr[kp + 1]; ++q) {
    const int i = qrow[q];
    const double w = qval[q];
    for (int e = brp[i]; e < brp[i + 1]; ++e) {
      const int k = bcol[e];
      if ((k & 31) != lane) continue;
      const double t = w * bval[e];
      const int s = acc.slot(k);
      if (s < 0) bad = true;
      else acc.val[s] += t;
    }
  }
  if (__any_sync(0xffffffffu, bad)) {
    if (lane == 0) atomicCAS(flag, 0, AF_SLOTS);
    return;
  }
  __syncwarp();
  const int total = emit_row(acc, lane, fill ? ocol + optr[kp] : nullptr, fill ? oval + optr[kp] : nullptr, fill);
  if (!fill && lane == 0) cnt[kp] = total;
}

// --------------------------------------------------------- transpose ----
__global__ void k_col_count(int n, const int* __restrict__ prp, const int* __restrict__ pcol, int* __restrict__ cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int e = prp[i]; e < prp[i + 1]; ++e) atomicAdd(&cnt[pcol[e]], 1);
}

__global__ void k_col_fill(int n, const int* __restrict__ prp, const int* __restrict__ pcol,
                           const double* __restrict__ pval, int* __restrict__ cursor, int* __restrict__ qrow,
                           double* __restrict__ qval) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int e = prp[i]; e < prp[i + 1]; ++e) {
    const int pos = atomicAdd(&cursor[pcol[e]], 1);
    qrow[pos] = i;
    qval[pos] = pval[e];
  }
}

// rows of each column in ascending order (CompColMatrix construct sorts them)
__global__ void k_col_sort(int c, const int* __restrict__ qptr, int* __restrict__ qrow, double* __restrict__ qval) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= c) return;
  for (int a = qptr[k] + 1; a < qptr[k + 1]; ++a) {
    const int r = qrow[a];
    const double v = qval[a];
    int b = a - 1;
    while (b >= qptr[k] && qrow[b] > r) {
      qrow[b + 1] = qrow[b];
      qval[b + 1] = qval[b];
      --b;
    }
    qrow[b + 1] = r;
    qval[b + 1] = v;
  }
}

// exclusive prefix sum of cnt[0..n) into ptr[0..n], one CTA
__global__ void __launch_bounds__(1024) k_scan(int n, const int* __restrict__ cnt, int* __restrict__ ptr) {
  __shared__ int part[1024];
  const int per = (n + 1023) / 1024;
  const int b0 = threadIdx.x * per, b1 = min(n, b0 + per);
  int s = 0;
  for (int i = b0; i < b1; ++i) s += cnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < 1024; ++t) {
      const int v = part[t];
      part[t] = run;
      run += v;
    }
    ptr[n] = run;
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int i = b0; i < b1; ++i) {
    ptr[i] = run;
    run += cnt[i];
  }
}

// ------------------------------------------------------------ coarsest ----
// DenseMatrix copy of the coarsest operator and dgetf2 (DenseLU.factor)
__global__ void k_dense_lu(int n, const int* __restrict__ rp, const int* __restrict__ col,
                           const double* __restrict__ val, double* __restrict__ A, int* __restrict__ piv,
                           int* __restrict__ info) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int q = 0; q < n * n; ++q) A[q] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int q = rp[i]; q < rp[i + 1]; ++q) A[i + col[q] * n] = val[q];
  int inf = 0;
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = fabs(A[j + j * n]);
    for (int i = j + 1; i < n; ++i) {
      const double a = fabs(A[i + j * n]);
      if (a > amax) {
        amax = a;
        jp = i;
      }
    }
    piv[j] = jp;
    if (A[jp + j * n] != 0.0) {
      if (jp != j)
        for (int c = 0; c < n; ++c) {
          const double t = A[j + c * n];
          A[j + c * n] = A[jp + c * n];
          A[jp + c * n] = t;
        }
      if (j < n - 1) {
        const double rcp = 1.0 / A[j + j * n];
        for (int i = j + 1; i < n; ++i) A[i + j * n] *= rcp;
      }
    } else if (inf == 0) {
      inf = j + 1;
    }
    if (j < n - 1)
      for (int c = j + 1; c < n; ++c) {
        const double yv = A[j + c * n];
        if (yv != 0.0) {
          const double temp = -1.0 * yv;
          for (int i = j + 1; i < n; ++i) A[i + c * n] += A[i + j * n] * temp;
        }
      }
  }
  *info = inf;
}

// directSolve (AMG.java:315-323): u = f, then dgetrs ('N' or 'T')
__global__ void k_dense_solve(int n, const double* __restrict__ A, const int* __restrict__ piv,
                              const double* __restrict__ f, double* __restrict__ u, int trans, const int* active) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (active && *active != 0) return;
  for (int i = 0; i < n; ++i) u[i] = f[i];
  if (!trans) {
    for (int j = 0; j < n; ++j)
      if (piv[j] != j) {
        const double t = u[j];
        u[j] = u[piv[j]];
        u[piv[j]] = t;
      }
    for (int k = 0; k < n; ++k)
      if (u[k] != 0.0)
        for (int i = k + 1; i < n; ++i) u[i] -= u[k] * A[i + k * n];
    for (int k = n - 1; k >= 0; --k)
      if (u[k] != 0.0) {
        u[k] = u[k] / A[k + k * n];
        for (int i = 0; i < k; ++i) u[i] -= u[k] * A[i + k * n];
      }
    return;
  }
  for (int i = 0; i < n; ++i) {
    double temp = u[i];
    for (int k = 0; k < i; ++k) temp -= A[k + i * n] * u[k];
    u[i] = temp / A[i + i * n];
  }
  for (int i = n - 1; i >= 0; --i) {
    double temp = u[i];
    for (int k = i + 1; k < n; ++k) temp -= A[k + i * n] * u[k];
    u[i] = temp;
  }
  for (int j = n - 1; j >= 0; --j)
    if (piv[j] != j) {
      const double t = u[j];
      u[j] = u[piv[j]];
      u[piv[j]] = t;
    }
}

// ------------------------------------------------------------- V-cycle ----
// Templated on the value type: double is the MTJ V-cycle, float the
// mixed-precision solver's FP32 copy of it (same order of operations).
// r = f; A.multAdd(-1, u, r) (CompRowMatrix.java:335-353)
template <typename T>
__global__ void k_amg_resid(int n, const int* __restrict__ rp, const int* __restrict__ col,
                            const T* __restrict__ val, const T* __restrict__ u, const T* __restrict__ f,
                            T* __restrict__ r, const int* active) {
  if (active && *active != 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T d = 0;
  for (int q = rp[i]; q < rp[i + 1]; ++q) d += val[q] * u[col[q]];
  r[i] = f[i] + (T)-1 * d;
}

// I.transMult(r, f_next) (CompColMatrix.java:299-316)
template <typename T>
__global__ void k_amg_restrict(int c, const int* __restrict__ qptr, const int* __restrict__ qrow,
                               const T* __restrict__ qval, const T* __restrict__ r, T* __restrict__ f,
                               const int* active) {
  if (active && *active != 0) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= c) return;
  T dot = 0;
  for (int q = qptr[j]; q < qptr[j + 1]; ++q) dot += qval[q] * r[qrow[q]];
  f[j] = dot;
}

// I.multAdd(u_next, u) (CompColMatrix.java:277-296, alpha 1): each row
// receives its terms in ascending column order
template <typename T>
__global__ void k_amg_prolong(int n, const int* __restrict__ prp, const int* __restrict__ pcol,
                              const T* __restrict__ pval, const T* __restrict__ un, T* __restrict__ u,
                              const int* active) {
  if (active && *active != 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T y = u[i];
  for (int e = prp[i]; e < prp[i + 1]; ++e) y += pval[e] * un[pcol[e]];
  u[i] = y;
}

template <typename A, typename B>
__global__ void k_amg_copy(int n, const A* __restrict__ a, B* __restrict__ b, const int* active) {
  if (active && *active != 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (B)a[i];
}

template <typename T>
__global__ void k_amg_zero(int n, T* __restrict__ b, const int* active) {
  if (active && *active != 0) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = 0;
}

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

int read_int(Context& ctx, const int* d) {
  int h = 0;
  RSG_CUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
  ctx.sync();
  return h;
}

// --------------------------------------------------------------- levels ----
struct AmgLevel {
  Csr* A = nullptr;           // operator of this level (owned below except on level 0)
  std::unique_ptr<Csr> own;
  DeviceBuffer<double> a0val; // level 0: the values at setup (AMG copies the matrix)
  const double* val = nullptr;
  int c = 0;                  // coarse size
  DeviceBuffer<int> pt, prp, pcol, qptr, qrow;
  DeviceBuffer<double> pval, qval;
  std::unique_ptr<Precond> smoother;  // SSOR, omegas switched between pre and post
  DeviceBuffer<double> u, f, r;
  // FP32 copies for the mixed-precision solver: operator, interpolation both ways, work vectors
  DeviceBuffer<float> valf, pvalf, qvalf, uf, ff, rf;
};

}  // namespace

struct AMGPrecond : Precond {
  Context* ctx;
  std::vector<AmgLevel> L;
  const int* pattern_id = nullptr;
  Csr* A0 = nullptr;
  int nc = 0, info = 0;
  DeviceBuffer<double> lu;
  DeviceBuffer<int> piv, dinfo, flag, counter;
  bool trans = false;
  explicit AMGPrecond(Context* c) : ctx(c) {}

  // Aggregator + Interpolator for level k; false when no aggregate formed
  bool coarsen(AmgLevel& lv, double eps, AmgLevel& next) {
    Context& c = *ctx;
    Csr& A = *lv.A;
    const int n = A.n, nnz = A.nnz;
    // Aggregator.findDiagonalIndices (AMG.java:446-461)
    for (int i = 0; i < n; ++i)
      if (A.h_diag[i] < 0)
        throw Error(RSG_MISSING_DIAGONAL, "Matrix is missing a diagonal entry on row " + std::to_string(i + 1));
    const int eb = blocks_for(n, 256);
    DeviceBuffer<unsigned char> S(std::max(nnz, 1)), R0(n), free2(n);
    DeviceBuffer<int> a1(n), a2(n), a3(n);
    flag.resize(1);
    counter.resize(1);
    RSG_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), c.stream));
    RSG_LAUNCH(c, "amg_strength", k_strength, eb, 256, 0, n, A.rowptr.get(), A.col.get(), lv.val, A.diag.get(), eps,
               S.get(), R0.get());
    // createInitialAggregates
    const size_t stage = sizeof(int) * (PHASE_CHUNK + 1) + (sizeof(int) + 1) * (size_t)PHASE_ENTRIES;
    const size_t bitmap = sizeof(unsigned) * (size_t)((n + 31) / 32);
    DeviceBuffer<unsigned> gbits;
    size_t smem = stage + bitmap;
    if (smem > 200 * 1024) {
      gbits.resize((n + 31) / 32);
      smem = stage;
    }
    static std::once_flag attr;
    std::call_once(attr, [] { cudaFuncSetAttribute(k_agg_greedy, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
    RSG_CUDA(cudaMemsetAsync(counter.get(), 0, sizeof(int), c.stream));
    PhaseArgs p1{n, A.rowptr.get(), A.col.get(), S.get(), R0.get(), nullptr, a1.get(), counter.get(), gbits.get(),
                 flag.get(), 0};
    RSG_LAUNCH(c, "amg_aggregate", k_agg_greedy, 1, 1024, smem, p1);
    // enlargeAggregates
    RSG_LAUNCH(c, "amg_enlarge", k_agg_enlarge, eb, 256, 0, n, A.rowptr.get(), A.col.get(), S.get(), R0.get(),
               a1.get(), a2.get(), free2.get(), flag.get());
    // createFinalAggregates (ids continue after the first phase's)
    PhaseArgs p3{n, A.rowptr.get(), A.col.get(), S.get(), free2.get(), nullptr, a3.get(), counter.get(), gbits.get(),
                 flag.get(), 1};
    RSG_LAUNCH(c, "amg_aggregate", k_agg_greedy, 1, 1024, smem, p3);
    const int cc = read_int(c, counter.get());
    if (read_int(c, flag.get())) throw Error(RSG_UNSUPPORTED, "AMG aggregation: a row has too many neighbours");
    if (cc == 0) return false;
    lv.c = cc;
    lv.pt.resize(n);
    RSG_LAUNCH(c, "amg_pt", k_agg_final, eb, 256, 0, n, a1.get(), a2.get(), a3.get(), lv.pt.get());
    // smoothed prolongation P (n x c), rows in ascending column order
    const int wb = blocks_for(n, AMG_WARPS);
    DeviceBuffer<int> cnt(std::max(n, cc) + 1);
    lv.prp.resize(n + 1);
    RSG_LAUNCH(c, "amg_prolong", k_prolong, wb, AMG_WARPS * 32, 0, n, A.rowptr.get(), A.col.get(), lv.val,
               A.diag.get(), S.get(), lv.pt.get(), AMG_OMEGA, 0, cnt.get(), nullptr, nullptr, nullptr, flag.get());
    RSG_LAUNCH(c, "amg_scan", k_scan, 1, 1024, 0, n, cnt.get(), lv.prp.get());
    const int pn = read_int(c, lv.prp.get() + n);
    lv.pcol.resize(std::max(pn, 1));
    lv.pval.resize(std::max(pn, 1));
    RSG_LAUNCH(c, "amg_prolong", k_prolong, wb, AMG_WARPS * 32, 0, n, A.rowptr.get(), A.col.get(), lv.val,
               A.diag.get(), S.get(), lv.pt.get(), AMG_OMEGA, 1, cnt.get(), lv.prp.get(), lv.pcol.get(),
               lv.pval.get(), flag.get());
    RSG_LAUNCH(c, "amg_sort", k_row_sort, eb, 256, 0, n, lv.prp.get(), lv.pcol.get(), lv.pval.get());
    // the same operator by columns (CompColMatrix)
    lv.qptr.resize(cc + 1);
    lv.qrow.resize(std::max(pn, 1));
    lv.qval.resize(std::max(pn, 1));
    RSG_CUDA(cudaMemsetAsync(cnt.get(), 0, sizeof(int) * (cc + 1), c.stream));
    RSG_LAUNCH(c, "amg_transpose", k_col_count, eb, 256, 0, n, lv.prp.get(), lv.pcol.get(), cnt.get());
    RSG_LAUNCH(c, "amg_scan", k_scan, 1, 1024, 0, cc, cnt.get(), lv.qptr.get());
    RSG_CUDA(cudaMemcpyAsync(cnt.get(), lv.qptr.get(), sizeof(int) * cc, cudaMemcpyDeviceToDevice, c.stream));
    RSG_LAUNCH(c, "amg_transpose", k_col_fill, eb, 256, 0, n, lv.prp.get(), lv.pcol.get(), lv.pval.get(), cnt.get(),
               lv.qrow.get(), lv.qval.get());
    RSG_LAUNCH(c, "amg_transpose", k_col_sort, blocks_for(cc, 128), 128, 0, cc, lv.qptr.get(), lv.qrow.get(),
               lv.qval.get());
    // B = A*P
    DeviceBuffer<int> brp(n + 1);
    RSG_LAUNCH(c, "amg_galerkin", k_galerkin_ap, wb, AMG_WARPS * 32, 0, n, A.rowptr.get(), A.col.get(), lv.val,
               lv.prp.get(), lv.pcol.get(), lv.pval.get(), 0, cnt.get(), nullptr, nullptr, nullptr, flag.get());
    RSG_LAUNCH(c, "amg_scan", k_scan, 1, 1024, 0, n, cnt.get(), brp.get());
    const int bn = read_int(c, brp.get() + n);
    DeviceBuffer<int> bcol(std::max(bn, 1));
    DeviceBuffer<double> bval(std::max(bn, 1));
    RSG_LAUNCH(c, "amg_galerkin", k_galerkin_ap, wb, AMG_WARPS * 32, 0, n, A.rowptr.get(), A.col.get(), lv.val,
               lv.prp.get(), lv.pcol.get(), lv.pval.get(), 1, cnt.get(), brp.get(), bcol.get(), bval.get(),
               flag.get());
    RSG_LAUNCH(c, "amg_sort", k_row_sort, eb, 256, 0, n, brp.get(), bcol.get(), bval.get());
    // Ac = P'*B
    const int cb = blocks_for(cc, AMG_WARPS);
    DeviceBuffer<int> arp(cc + 1);
    RSG_LAUNCH(c, "amg_galerkin", k_galerkin_ptb, cb, AMG_WARPS * 32, 0, cc, lv.qptr.get(), lv.qrow.get(),
               lv.qval.get(), brp.get(), bcol.get(), bval.get(), 0, cnt.get(), nullptr, nullptr, nullptr, flag.get());
    RSG_LAUNCH(c, "amg_scan", k_scan, 1, 1024, 0, cc, cnt.get(), arp.get());
    const int an = read_int(c, arp.get() + cc);
    DeviceBuffer<int> acol(std::max(an, 1));
    DeviceBuffer<double> aval(std::max(an, 1));
    RSG_LAUNCH(c, "amg_galerkin", k_galerkin_ptb, cb, AMG_WARPS * 32, 0, cc, lv.qptr.get(), lv.qrow.get(),
               lv.qval.get(), brp.get(), bcol.get(), bval.get(), 1, cnt.get(), arp.get(), acol.get(), aval.get(),
               flag.get());
    RSG_LAUNCH(c, "amg_sort", k_row_sort, blocks_for(cc, 256), 256, 0, cc, arp.get(), acol.get(), aval.get());
    if (read_int(c, flag.get())) throw Error(RSG_UNSUPPORTED, "AMG setup: a row of P, A*P or P'AP has too many columns");
    // the coarse operator as a CompRowMatrix
    std::vector<int> hrp(cc + 1), hcol(std::max(an, 1));
    RSG_CUDA(cudaMemcpyAsync(hrp.data(), arp.get(), sizeof(int) * (cc + 1), cudaMemcpyDeviceToHost, c.stream));
    RSG_CUDA(cudaMemcpyAsync(hcol.data(), acol.get(), sizeof(int) * std::max(an, 1), cudaMemcpyDeviceToHost,
                             c.stream));
    c.sync();
    next.own.reset(new Csr());
    next.own->build(ctx, cc, an, hrp.data(), hcol.data());
    if (an) RSG_CUDA(cudaMemcpyAsync(next.own->val.get(), aval.get(), sizeof(double) * an, cudaMemcpyDeviceToDevice,
                                     c.stream));
    next.own->sell_dirty = true;
    next.A = next.own.get();
    next.val = next.own->val.get();
    c.sync();
    return true;
  }

  void setup(Csr& M) override {
    // AMG.setMatrix (AMG.java:224-286)
    Context& c = *ctx;
    f32_ready = false;
    for (int k = 0; k < M.n; ++k)
      if (M.h_diag[k] < 0)
        throw Error(RSG_MISSING_DIAGONAL, "Matrix is missing a diagonal entry on row " + std::to_string(k + 1));
    L.clear();
    L.emplace_back();
    L[0].A = &M;
    L[0].a0val.resize(std::max(M.nnz, 1));
    RSG_CUDA(cudaMemcpyAsync(L[0].a0val.get(), M.val.get(), sizeof(double) * std::max(M.nnz, 1),
                             cudaMemcpyDeviceToDevice, c.stream));
    L[0].val = L[0].a0val.get();
    A0 = &M;
    for (int k = 0; L[k].A->n > AMG_MIN; ++k) {
      const double eps = 0.08 * std::pow(0.5, k);
      AmgLevel next;
      if (!coarsen(L[k], eps, next)) break;
      L.push_back(std::move(next));
    }
    const int m = (int)L.size();
    for (int k = 0; k < m; ++k) {
      const int n = L[k].A->n;
      L[k].u.resize(n);
      L[k].f.resize(n);
      L[k].r.resize(n);
      RSG_CUDA(cudaMemsetAsync(L[k].u.get(), 0, sizeof(double) * n, c.stream));
      if (k < m - 1) {
        L[k].smoother = make_precond(ctx, RSG_PC_SSOR);
        L[k].smoother->setup(*L[k].A);  // SSOR.setMatrix copies the values
      }
    }
    // DenseLU of the coarsest operator
    Csr& Ac = *L[m - 1].A;
    nc = Ac.n;
    if (nc > COARSE_MAX)
      throw Error(RSG_UNSUPPORTED, "AMG coarsening stopped at " + std::to_string(nc) +
                                       " rows; the dense coarsest solve takes at most " + std::to_string(COARSE_MAX));
    lu.resize((size_t)nc * nc);
    piv.resize(nc);
    dinfo.resize(1);
    RSG_LAUNCH(c, "amg_dense_lu", k_dense_lu, 1, 32, 0, nc, Ac.rowptr.get(), Ac.col.get(), L[m - 1].val, lu.get(),
               piv.get(), dinfo.get());
    info = read_int(c, dinfo.get());
  }

  void cycle(int k, const int* active) {
    // AMG.java:288-313
    Context& c = *ctx;
    const int m = (int)L.size();
    AmgLevel& l = L[k];
    const int n = l.A->n;
    if (k == m - 1) {
      if (info > 0) throw Error(RSG_SINGULAR, "MatrixSingularException: the coarsest AMG operator is singular");
      RSG_LAUNCH(c, "amg_direct", k_dense_solve, 1, 32, 0, nc, lu.get(), piv.get(), l.f.get(), l.u.get(),
                 trans ? 1 : 0, active);
      return;
    }
    AmgLevel& nx = L[k + 1];
    const int eb = blocks_for(n, 256);
    set_ssor_params(l.smoother.get(), 1.0, 1.85, 1);  // preRelax: SSOR(omegaPreF, omegaPreR)
    l.smoother->apply(l.f.get(), l.u.get(), active);
    RSG_LAUNCH(c, "amg_zero", k_amg_zero<double>, blocks_for(nx.A->n, 256), 256, 0, nx.A->n, nx.u.get(), active);
    RSG_LAUNCH(c, "amg_resid", k_amg_resid<double>, eb, 256, 0, n, l.A->rowptr.get(), l.A->col.get(), l.val,
               l.u.get(), l.f.get(), l.r.get(), active);
    RSG_LAUNCH(c, "amg_restrict", k_amg_restrict<double>, blocks_for(l.c, 256), 256, 0, l.c, l.qptr.get(),
               l.qrow.get(), l.qval.get(), l.r.get(), nx.f.get(), active);
    cycle(k + 1, active);
    RSG_LAUNCH(c, "amg_prolong", k_amg_prolong<double>, eb, 256, 0, n, l.prp.get(), l.pcol.get(), l.pval.get(),
               nx.u.get(), l.u.get(), active);
    set_ssor_params(l.smoother.get(), 1.85, 1.0, 1);  // postRelax: SSOR(omegaPostF, omegaPostR)
    l.smoother->apply(l.f.get(), l.u.get(), active);
  }

  void run(const double* b, double* x, const int* active, bool t) {
    // apply / transApply (AMG.java:208-222): u0 = x, f0 = b, cycle, x = u0
    Context& c = *ctx;
    const int n = L[0].A->n;
    const int eb = blocks_for(n, 256);
    RSG_LAUNCH(c, "amg_copy", (k_amg_copy<double, double>), eb, 256, 0, n, x, L[0].u.get(), active);
    RSG_LAUNCH(c, "amg_copy", (k_amg_copy<double, double>), eb, 256, 0, n, b, L[0].f.get(), active);
    trans = t;
    cycle(0, active);
    RSG_LAUNCH(c, "amg_copy", (k_amg_copy<double, double>), eb, 256, 0, n, L[0].u.get(), x, active);
  }

  // FP32 copy of the hierarchy, made on the first FP32 apply after a setup:
  // operators, interpolation and the smoothers' coefficients in FP32 (half
  // the bytes per V-cycle); the coarsest LU stays FP64.
  bool f32_ready = false;
  void build_f32() {
    Context& c = *ctx;
    const int m = (int)L.size();
    for (int k = 0; k < m; ++k) {
      AmgLevel& l = L[k];
      const int64_t nnz = std::max(l.A->nnz, 1), n = l.A->n;
      l.valf.resize(nnz);
      RSG_LAUNCH(c, "amg_f32", k_to_f32, blocks_for(nnz, 256), 256, 0, nnz, l.val, l.valf.get());
      if (k < m - 1) {
        const int64_t pn = (int64_t)l.pval.size();
        l.pvalf.resize(pn);
        l.qvalf.resize(pn);
        RSG_LAUNCH(c, "amg_f32", k_to_f32, blocks_for(pn, 256), 256, 0, pn, l.pval.get(), l.pvalf.get());
        RSG_LAUNCH(c, "amg_f32", k_to_f32, blocks_for(pn, 256), 256, 0, pn, l.qval.get(), l.qvalf.get());
      }
      l.uf.resize(n);
      l.ff.resize(n);
      l.rf.resize(n);
    }
    f32_ready = true;
  }

  void cycle_f32(int k, const int* active) {
    Context& c = *ctx;
    const int m = (int)L.size();
    AmgLevel& l = L[k];
    const int n = l.A->n;
    const int eb = blocks_for(n, 256);
    if (k == m - 1) {
      if (info > 0) throw Error(RSG_SINGULAR, "MatrixSingularException: the coarsest AMG operator is singular");
      RSG_LAUNCH(c, "amg_coarse_cvt", (k_amg_copy<float, double>), eb, 256, 0, n, l.ff.get(), l.f.get(), active);
      RSG_LAUNCH(c, "amg_direct", k_dense_solve, 1, 32, 0, nc, lu.get(), piv.get(), l.f.get(), l.u.get(), 0, active);
      RSG_LAUNCH(c, "amg_coarse_cvt", (k_amg_copy<double, float>), eb, 256, 0, n, l.u.get(), l.uf.get(), active);
      return;
    }
    AmgLevel& nx = L[k + 1];
    set_ssor_params(l.smoother.get(), 1.0, 1.85, 1);
    l.smoother->apply_f32(l.ff.get(), l.uf.get(), active);
    RSG_LAUNCH(c, "amg_zero", k_amg_zero<float>, blocks_for(nx.A->n, 256), 256, 0, nx.A->n, nx.uf.get(), active);
    RSG_LAUNCH(c, "amg_resid", k_amg_resid<float>, eb, 256, 0, n, l.A->rowptr.get(), l.A->col.get(), l.valf.get(),
               l.uf.get(), l.ff.get(), l.rf.get(), active);
    RSG_LAUNCH(c, "amg_restrict", k_amg_restrict<float>, blocks_for(l.c, 256), 256, 0, l.c, l.qptr.get(),
               l.qrow.get(), l.qvalf.get(), l.rf.get(), nx.ff.get(), active);
    cycle_f32(k + 1, active);
    RSG_LAUNCH(c, "amg_prolong", k_amg_prolong<float>, eb, 256, 0, n, l.prp.get(), l.pcol.get(), l.pvalf.get(),
               nx.uf.get(), l.uf.get(), active);
    set_ssor_params(l.smoother.get(), 1.85, 1.0, 1);
    l.smoother->apply_f32(l.ff.get(), l.uf.get(), active);
  }

  // One FP32 V-cycle from a zero start (the inner stage of the mixed-precision
  // solver wants a fixed linear preconditioner, unlike MTJ's apply, which
  // starts from the caller's vector).
  void apply_f32(const float* b, float* x, const int* active) override {
    Context& c = *ctx;
    if (!f32_ready) build_f32();
    const int n = L[0].A->n;
    const int eb = blocks_for(n, 256);
    RSG_LAUNCH(c, "amg_zero", k_amg_zero<float>, eb, 256, 0, n, L[0].uf.get(), active);
    RSG_LAUNCH(c, "amg_copy", (k_amg_copy<float, float>), eb, 256, 0, n, b, L[0].ff.get(), active);
    cycle_f32(0, active);
    RSG_LAUNCH(c, "amg_copy", (k_amg_copy<float, float>), eb, 256, 0, n, L[0].uf.get(), x, active);
  }

  void apply(const double* b, double* x, const int* active) override { run(b, x, active, false); }
  void trans_apply(const double* b, double* x, const int* active) override { run(b, x, active, true); }

  // hierarchy export for the parity tests
  int levels() const { return (int)L.size(); }
};

std::unique_ptr<Precond> make_amg(Context* ctx) { return std::unique_ptr<Precond>(new AMGPrecond(ctx)); }

// sizes: n, nnz, c, nnz(P)
void amg_level_sizes(Precond* p, int k, int* sizes) {
  auto* a = dynamic_cast<AMGPrecond*>(p);
  if (!a) throw Error(RSG_BAD_ARG, "solver does not use AMG");
  if (k < 0 || k >= a->levels()) throw Error(RSG_BAD_ARG, "no such AMG level");
  AmgLevel& l = a->L[k];
  sizes[0] = l.A->n;
  sizes[1] = l.A->nnz;
  sizes[2] = l.c;
  int pn = 0;
  if (l.c) {
    RSG_CUDA(cudaMemcpy(&pn, l.prp.get() + l.A->n, sizeof(int), cudaMemcpyDeviceToHost));
  }
  sizes[3] = pn;
}

int amg_levels(Precond* p) {
  auto* a = dynamic_cast<AMGPrecond*>(p);
  if (!a) throw Error(RSG_BAD_ARG, "solver does not use AMG");
  return a->levels();
}

void amg_level_get(Precond* p, int k, int* rowptr, int* col, double* val, int* pt, int* colptr, int* rowind,
                   double* Idata) {
  auto* a = dynamic_cast<AMGPrecond*>(p);
  if (!a) throw Error(RSG_BAD_ARG, "solver does not use AMG");
  if (k < 0 || k >= a->levels()) throw Error(RSG_BAD_ARG, "no such AMG level");
  Context& c = *a->ctx;
  AmgLevel& l = a->L[k];
  const int n = l.A->n, nnz = l.A->nnz;
  auto get = [&](void* dst, const void* src, size_t bytes) {
    if (dst && bytes) RSG_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c.stream));
  };
  get(rowptr, l.A->rowptr.get(), sizeof(int) * (n + 1));
  get(col, l.A->col.get(), sizeof(int) * nnz);
  get(val, l.val, sizeof(double) * nnz);
  if (l.c) {
    int pn = 0;
    RSG_CUDA(cudaMemcpyAsync(&pn, l.prp.get() + n, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    get(pt, l.pt.get(), sizeof(int) * n);
    get(colptr, l.qptr.get(), sizeof(int) * (l.c + 1));
    get(rowind, l.qrow.get(), sizeof(int) * pn);
    get(Idata, l.qval.get(), sizeof(double) * pn);
  }
  c.sync();
}

}  // namespace rsg
