// Sparse linear algebra on the GPU: CompRowMatrix storage (CSR plus a
// SELL-32 copy for coalesced SpMV), deterministic reductions, level
// scheduled triangular sweeps (ILU(0), SSOR) and the Krylov drivers.
#pragma once
#include <memory>

#include "common.cuh"

namespace rsg {

constexpr int SELL_C = 32;

// One row of the SELL-32 copy (entry k of the row in lane l of slice s at
// slice_base[s] + 32 k + l) times x, each product fused into the running
// sum, in CSR order.  NC: x gathers through the read-only cache, for an x
// that no thread writes during the kernel; otherwise from L2 (an x written
// earlier in the same launch by other SMs, as in a persistent solver).
template <bool NC>
__device__ __forceinline__ double sell_row_fma(const double* __restrict__ val, const int* __restrict__ col,
                                               const double* x, int base, int len) {
  double d = 0;
#pragma unroll 8
  for (int k = 0; k < len; ++k) {
    const int q = base + 32 * k;
    const double xv = NC ? __ldg(x + col[q]) : __ldcg(x + col[q]);
    d = __fma_rn(val[q], xv, d);
  }
  return d;
}

// Ring schedule of an ILU(0) sweep for one cluster of C CTAs (precond.cu,
// k_sweep_ring): CTAs own contiguous row blocks, every level has
// RING_SLICES slices (W = RING_SLICES / C per CTA), each value is pushed only
// to the CTAs that read it.  R == 0: no ring schedule for this pattern.
struct RingPlan {
  int C = 0, nlev = 0, R = 0, slack = 0;
  int maxlen = 0;  // longest row (entries in the sweep's triangle)
  DeviceBuffer<int> slice_base, row, len, ridx, src, diag_src, expect;
  DeviceBuffer<unsigned short> pmask, nbr;
  DeviceBuffer<double> val, diag;
  DeviceBuffer<float> valf, diagf;
};

// Level schedule of a triangular sweep, laid out as SELL-32 slices that never
// straddle a level: slot (slice s, lane l, k) lives at base[s] + 32*k + l.
struct SweepPlan {
  int nlev = 0, nslices = 0;
  std::vector<int> h_level_slices;  // nlev + 1 slice offsets
  DeviceBuffer<int> level_slices, slice_base, slice_width, row, len, col, src;
  DeviceBuffer<double> val;   // FP64 coefficients (gathered from CSR via src)
  DeviceBuffer<float> valf;   // FP32 copy for the mixed-precision inner solver
  DeviceBuffer<int> diag_src; // CSR position of each slot row's diagonal (upper sweeps)
  DeviceBuffer<double> diag;  // diagonal per slot row (upper sweeps)
  DeviceBuffer<float> diagf;
  int max_rows_per_level = 0;
  // ILU sweeps only: ring schedules for clusters of 16 CTAs (4 warps each)
  // and of 8 CTAs (8 warps each); pick[0] / pick[1] is the one the walk
  // autotuner chose for the FP64 / FP32 values (R == 0: no schedule)
  RingPlan rings[2];
  int pick[2] = {0, 0};
  bool tuned = false;
  const RingPlan& ring(int prec) const { return rings[pick[prec]]; }
};

constexpr int RING_SLICES = 64;

struct Csr {
  Context* ctx = nullptr;
  int n = 0, nnz = 0;
  std::vector<int> h_rowptr, h_col;
  DeviceBuffer<int> rowptr, col;
  DeviceBuffer<double> val;
  // SELL-32 copy used by SpMV
  int nslices = 0;
  int64_t sell_size = 0;
  DeviceBuffer<int> slice_base, row_len, sell_col, sell_src;
  DeviceBuffer<double> sell_val;
  DeviceBuffer<float> sell_valf;
  bool sell_dirty = true;
  // diagonal positions (-1 if missing)
  std::vector<int> h_diag;
  DeviceBuffer<int> diag;
  void build(Context* c, int n, int nnz, const int* rowptr, const int* col);
  void refresh_sell();   // gathers CSR values into the SELL copy if stale
  void refresh_sell_f32();
};

// Device-resident scalar state of one Krylov solve.
struct KState {
  double rho_1, rho_2, alpha, beta, omega, rho;
  double residual, initR;
  double rtol, atol, dtol;
  double vscale;  // GMRES 1/H(i+1,i)
  int iter, maxIter;
  int status;     // 0 running, 1 converged, 2 converged on s (BiCGstab), negative: rsg_status failure
  int first;
  int hist_len, hist_cap;
  int gm_i;       // GMRES inner index
  int gm_exit;    // GMRES inner loop finished
  int restart;
  int inner;      // mixed precision: inner iterations summed over outer steps
};

enum { KS_RUNNING = 0, KS_CONVERGED = 1, KS_CONVERGED_S = 2 };

struct Precond {
  virtual ~Precond() {}
  virtual void setup(Csr& A) = 0;
  // x := M^{-1} b (x may be read as the starting iterate, as SSOR does)
  virtual void apply(const double* b, double* x, const int* active) = 0;
  virtual void trans_apply(const double* b, double* x, const int* active) = 0;
  // Preconditioner.apply with MTJ's rounding (the solvers' applies may fuse
  // multiply-adds)
  virtual void apply_exact(const double* b, double* x) { apply(b, x, nullptr); }
  // FP32 variant for the mixed-precision inner solver
  virtual void apply_f32(const float* b, float* x, const int* active) {
    throw Error(RSG_UNSUPPORTED, "preconditioner has no FP32 variant");
  }
};

std::unique_ptr<Precond> make_precond(Context* ctx, int kind);
std::unique_ptr<Precond> make_amg(Context* ctx);  // amg.cu
int amg_levels(Precond* p);
void amg_level_sizes(Precond* p, int k, int* sizes);
void amg_level_get(Precond* p, int k, int* rowptr, int* col, double* val, int* pt, int* colptr, int* rowind,
                   double* Idata);

// Krylov solver handle (defined in krylov.cu)
struct Solver;
struct SolverDeleter {
  void operator()(Solver* s) const;
};
using SolverPtr = std::unique_ptr<Solver, SolverDeleter>;
SolverPtr make_solver(Context* ctx, int method, int precond, double rtol, double atol, double dtol, int maxit,
                      int restart);
void solver_setup(Solver& s, Csr& A);
void solver_solve(Solver& s, Csr& A, const double* b, double* x, rsg_solve_info* info);
void solver_set_inner(Solver& s, int iterations, double rtol);
// what a solver was created with, and its preconditioner
struct SolverView {
  int method, pc_kind;
  Precond* pc;
  double rtol, atol, dtol;
  int maxIter;
  const Csr* setup_for;  // the matrix of the last setup (nullptr: none)
  Context* ctx;
  int restart;          // GMRES restart (default 30)
  int inner_iters;      // mixed precision: FP32 inner BiCGstab steps per outer step
  double inner_rtol;
};
SolverView solver_view(Solver& s);
// One pressure system of an ensemble member: A x = b with the member's
// solver (BiCGstab + ILU(0), set up on A), on the member's context.
struct EnsSystem {
  Context* ctx;
  Csr* A;
  Solver* solver;
  const double* b;
  double* x;
};
// Solves every system in one persistent launch (ensemble.cu).  precision 0:
// FP64 ILU(0) walks, 1: the factors' FP32 copies inside the FP64 BiCGstab.
// status[i]: RSG_OK or the member's failure (MTJ's reasons, RSG_TIMEOUT).
void ensemble_solve(const std::vector<EnsSystem>& sys, int precision, std::vector<rsg_solve_info>& info,
                    std::vector<int>& status);
// the ring schedules and factor values of an ILU(0) preconditioner after its
// setup, for clusters of `prefer` CTAs when planned, else the other shape
// (false for other preconditioners or patterns without ring schedules)
bool ilu_ring_plans(Precond* p, int prefer, const RingPlan** lower, const RingPlan** upper);
// walk autotuner of an ILU(0) preconditioner: force >= 0 sets the cluster
// shape (0: timed choice, 16 or 8 CTAs), applied at the next setup; shapes
// (when given) receives the clusters in use: FP64 lower, upper, FP32 lower,
// upper (0: no ring schedule).  false for other preconditioners.
bool ilu_walk_shape(Precond* p, int force, int* shapes);
// the solver no longer refers to the matrix of its last setup (rsg_solver_setup is needed again)
void solver_forget_matrix(Solver& s);

// Explicit transpose of a CSR matrix with a fixed position map: the pattern
// of A^T is built on the host once per pattern of A, after which update()
// gathers A's current values into A^T with one kernel.
struct CsrTranspose {
  Csr AT;
  DeviceBuffer<int> src;  // AT.val[q] = A.val[src[q]]
  std::vector<int> for_rowptr, for_col;
  void update(Csr& A);
};

// Launches of BLAS-1 style kernels shared by the drivers.
void launch_spmv(Context& ctx, Csr& A, const double* x, double* y, const int* active);
void launch_spmv_f32(Context& ctx, Csr& A, const float* x, float* y, const int* active);

}  // namespace rsg

struct rsg_csr {
  rsg::Csr m;
};

struct rsg_solver {
  rsg::SolverPtr s;
};
