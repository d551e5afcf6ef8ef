/*
 * resgpu: GB300 (sm_103a) implementation of the RS reservoir simulator's
 * pressure hot path and of the MTJ sparse solver stack it calls.
 *
 * C ABI.  Plain pointers and sizes only; every call returns an rsg_status.
 * Host buffers passed in are caller owned and only read or written during
 * the call.  Device buffers are owned by the library and live behind the
 * opaque handles.  One context owns one CUDA stream; handles created from a
 * context must be used from one host thread at a time (MTJ solver objects
 * are not re-entrant either: mtj/src/no/uib/cipr/matrix/sparse/BiCGstab.java:42-63).
 * Destroy every handle created from a context before destroying the context.
 *
 * Reference interfaces replaced (paths relative to the RS/MTJ sources):
 *   rsg_csr_*      sparse/CompRowMatrix.java:160-190 (construct), :300-372
 *                  (mult/multAdd/transMult), :404-453 (add/zero)
 *   rsg_solver_*   sparse/IterativeSolver.java:43-74 (solve),
 *                  sparse/Preconditioner.java:42-63 (apply/setMatrix),
 *                  sparse/DefaultIterationMonitor.java:72-156 (tolerances)
 *   rsg_mesh_*     geometry/flux/TransmissibilityComputer.java:30-31
 *                  (calculateTransmissibilities), numerics/LinearSolver.java:111-168
 *                  (sparsity pattern)
 *   rsg_sim_*      numerics/Discretisation.java:208-225 (solve(dt)),
 *                  field/Field.java:69-96 (initialisation), :488-501
 *                  (calculateSecondaries)
 */
#ifndef RSG_H
#define RSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSG_ABI_VERSION 1
#define RSG_MAX_COMPONENTS 8

/* Status codes.  1..3 are MTJ's NotConvergedException.Reason values
 * (sparse/IterativeSolverNotConvergedException.java:29-91). */
typedef int32_t rsg_status;
enum {
  RSG_OK = 0,
  RSG_NOT_CONVERGED_ITERATIONS = 1,
  RSG_NOT_CONVERGED_DIVERGENCE = 2,
  RSG_NOT_CONVERGED_BREAKDOWN = 3,
  RSG_ZERO_PIVOT = 4,           /* sparse/ILU.java:105-107 */
  RSG_MISSING_DIAGONAL = 5,     /* sparse/ILU.java:134-136 */
  RSG_OUT_OF_PATTERN = 6,       /* sparse/CompRowMatrix.java:435 */
  RSG_NONPOSITIVE_PRESSURE = 7, /* numerics/Discretisation.java:349-351 */
  RSG_NEGATIVE_MOLES = 8,       /* numerics/Discretisation.java:800-812 */
  RSG_BAD_ARG = 9,
  RSG_CUDA_ERROR = 10,
  RSG_TIMEOUT = 11,
  RSG_UNSUPPORTED = 12,
  RSG_NEWTON_NOT_CONVERGED = 13, /* numerics/Discretisation.java:327-329 */
  RSG_SINGULAR = 14,             /* MatrixSingularException in MPFA / dense LU */
  RSG_PHYSICS = 15               /* field/CV.java:496-500 and EOS data checks */
};

/* Krylov methods (numerics/LinearSolver.java:173-191) */
enum { RSG_CG = 0, RSG_BICGSTAB = 1, RSG_GMRES = 2, RSG_FGMRES_MIXED = 3 };
/* Preconditioners (numerics/LinearSolver.java:197-221) */
enum { RSG_PC_NONE = 0, RSG_PC_DIAGONAL = 1, RSG_PC_ILU = 2, RSG_PC_SSOR = 3, RSG_PC_AMG = 4 };

typedef struct rsg_ctx rsg_ctx;
typedef struct rsg_csr rsg_csr;
typedef struct rsg_solver rsg_solver;
typedef struct rsg_mesh rsg_mesh;
typedef struct rsg_sim rsg_sim;

/* ------------------------------------------------------------ context -- */
int32_t rsg_abi_version(void);
const char* rsg_status_string(rsg_status s);
/* Creates a context on CUDA device `device` (fails loudly with
 * RSG_CUDA_ERROR when no sm_103 device is usable: there is no CPU path). */
rsg_status rsg_context_create(int32_t device, rsg_ctx** out);
rsg_status rsg_context_destroy(rsg_ctx* ctx);
/* Last error message recorded on the context (empty if none). */
const char* rsg_context_last_error(rsg_ctx* ctx);
/* How the level-scheduled triangular sweeps run in this process:
 * -1 not decided yet, 0 one launch per level, 1 one thread-block cluster
 * walking all levels with hardware cluster barriers, 2 ILU sweeps on one
 * cluster whose CTAs own contiguous row blocks and push each computed value
 * through distributed shared memory to the CTAs that read it (st.async +
 * mbarrier transaction counts, no cluster barrier per level). */
int32_t rsg_sweep_mode(void);
/* Builds on the host the distributed-shared-memory schedule of one ILU(0)
 * triangular sweep of a CSR pattern (sweep 0: the unit lower solve, 1: the
 * upper solve; ctas: 8 or 16 CTAs in the cluster) and checks it against the
 * pattern: every row placed once, every index inside its array, every
 * operand either computed in the reading CTA or pushed to it within the
 * ring's depth, and the per-level receive counts equal to the values pushed.
 * stats (4 values, may be NULL): plan levels, ring depth, values pushed in
 * one sweep, most neighbours of one CTA.  Needs no GPU.  Returns RSG_OK for a
 * sound schedule, RSG_UNSUPPORTED when the pattern has none (the sweep then
 * runs without the ring), RSG_OUT_OF_PATTERN when the check fails (msg, of
 * msg_len bytes, may be NULL, says what failed).  Inspection only: no
 * counterpart in the reference (UnitLowerCompRowMatrix.solve and
 * UpperCompRowMatrix.solve, mtj/src/no/uib/cipr/matrix/sparse/ILU.java:54-140,
 * are sequential loops). */
rsg_status rsg_sweep_plan_check(int32_t n, const int32_t* row_ptr, const int32_t* col, int32_t sweep, int32_t ctas,
                                int64_t* stats, char* msg, int32_t msg_len);
/* Number of kernels this context has launched so far. */
int64_t rsg_context_kernel_launches(rsg_ctx* ctx);
/* Waits for all work queued on the context's stream. */
rsg_status rsg_context_synchronize(rsg_ctx* ctx);
/* Kernel-time accounting: when enabled, the library brackets its kernels
 * with CUDA events on its own stream and accumulates per-kernel-family
 * device time.  names: '\n'-separated family names written into buf. */
rsg_status rsg_context_set_profiling(rsg_ctx* ctx, int32_t enabled);
rsg_status rsg_context_profile_read(rsg_ctx* ctx, int32_t max_entries, double* ms, int64_t* launches,
                                    char* names, int32_t names_len, int32_t* n_entries);
rsg_status rsg_context_profile_reset(rsg_ctx* ctx);
/* CUDA events on the context's stream for device-side timing: record into
 * one of 64 slots, then read the elapsed milliseconds between two slots. */
rsg_status rsg_context_timer_record(rsg_ctx* ctx, int32_t slot);
rsg_status rsg_context_timer_elapsed(rsg_ctx* ctx, int32_t slot_a, int32_t slot_b, double* ms);
/* Page-locked host memory for callers that stage inputs and results. */
rsg_status rsg_host_alloc(size_t bytes, void** ptr);
rsg_status rsg_host_free(void* ptr);

/* ----------------------------------------------- CompRowMatrix (CSR) -- */
/* Copies the pattern to the device.  Column indices must be sorted within
 * each row (CompRowMatrix.construct sorts them). */
rsg_status rsg_csr_create(rsg_ctx* ctx, int32_t n, int32_t nnz, const int32_t* row_ptr, const int32_t* col,
                          rsg_csr** out);
rsg_status rsg_csr_destroy(rsg_csr* A);
rsg_status rsg_csr_set_values(rsg_csr* A, const double* values); /* host, nnz */
rsg_status rsg_csr_get_values(rsg_csr* A, double* values);       /* host, nnz */
/* y = A x  (CompRowMatrix.mult); host vectors of length n. */
rsg_status rsg_csr_mult(rsg_csr* A, const double* x, double* y);
/* y = alpha A x + y  (CompRowMatrix.multAdd) */
rsg_status rsg_csr_mult_add(rsg_csr* A, double alpha, const double* x, double* y);
/* y = A^T x  (CompRowMatrix.transMult) */
rsg_status rsg_csr_trans_mult(rsg_csr* A, const double* x, double* y);
/* Matrices.zeroRows(A, diagonal, rows) (mtj/src/no/uib/cipr/matrix/Matrices.java:631-652) */
rsg_status rsg_csr_zero_rows(rsg_csr* A, double diagonal, int32_t nrows, const int32_t* rows);
/* Device pointers of the CSR arrays (for callers that keep vectors on the GPU). */
rsg_status rsg_csr_device_arrays(rsg_csr* A, const int32_t** row_ptr, const int32_t** col, double** values);

/* ------------------------------ IterativeSolver + Preconditioner -------- */
typedef struct {
  int32_t iterations;    /* IterationMonitor.iterations() at exit */
  int32_t reason;        /* rsg_status of the solve */
  double residual;       /* last monitored residual norm */
  double initial_residual;
  int32_t inner_iterations; /* FP32 inner iterations (mixed precision only) */
  int32_t refinements;      /* FP64 outer cycles (mixed precision only) */
} rsg_solve_info;

rsg_status rsg_solver_create(rsg_ctx* ctx, int32_t method, int32_t precond, rsg_solver** out);
rsg_status rsg_solver_destroy(rsg_solver* s);
/* DefaultIterationMonitor(maxIter, rtol, atol, dtol) */
rsg_status rsg_solver_set_monitor(rsg_solver* s, double rtol, double atol, double dtol, int32_t max_iter);
/* GMRES.setRestart (default 30) */
rsg_status rsg_solver_set_restart(rsg_solver* s, int32_t restart);
/* Mixed precision (RSG_FGMRES_MIXED): FP64 flexible GMRES(restart) whose
 * preconditioner is `inner_iterations` FP32 BiCGstab steps (stopping early at
 * inner_rtol) with the FP32 copy of the preconditioner: ILU(0) factors, or
 * the AMG hierarchy (operators, interpolation and SSOR smoother coefficients
 * in FP32, one V-cycle from a zero start per application, coarsest LU in
 * FP64), or the inverted diagonal.  SSOR is not offered.  Default 10, 1e-3.
 * No counterpart in the reference (a new capability beside MTJ's solvers). */
rsg_status rsg_solver_set_inner(rsg_solver* s, int32_t inner_iterations, double inner_rtol);
/* SSOR omegas (SSOR(F, reverse, omegaF, omegaR)) */
rsg_status rsg_solver_set_ssor(rsg_solver* s, double omega_f, double omega_r, int32_t reverse);
/* Preconditioner.setMatrix(A): ILU(0) factorisation / diagonal inversion. */
rsg_status rsg_solver_setup(rsg_solver* s, rsg_csr* A);
/* IterativeSolver.solve(A, b, x): x is the initial guess on entry and the
 * solution on exit (host arrays of length n). */
rsg_status rsg_solver_solve(rsg_solver* s, rsg_csr* A, const double* b, double* x, rsg_solve_info* info);
/* Level-walk shape of an ILU(0) solver (no counterpart in the reference).
 * The ILU(0) triangular solves walk the levels on one thread-block cluster,
 * planned for 16 CTAs of 4 warps and for 8 CTAs of 8 warps; the first setup on
 * a pattern times both on the factors and keeps the faster per sweep and per
 * precision (the walk autotuner).  Every shape gives the same bits.
 * rsg_solver_set_walk_shape(s, 16 or 8) fixes the shape, 0 returns to the
 * timed choice (applied at the next rsg_solver_setup); rsg_solver_walk_shapes
 * reports the clusters in use: FP64 lower, upper, FP32 lower, upper (0: no
 * cluster walk).  RSG_UNSUPPORTED for other preconditioners. */
rsg_status rsg_solver_set_walk_shape(rsg_solver* s, int32_t ctas);
rsg_status rsg_solver_walk_shapes(rsg_solver* s, int32_t* shapes);
/* The same for a simulator's pressure solver. */
rsg_status rsg_sim_walk_shapes(rsg_sim* s, int32_t* shapes);
/* Same with device-resident b and x (device pointers from this context). */
rsg_status rsg_solver_solve_device(rsg_solver* s, rsg_csr* A, const double* d_b, double* d_x, rsg_solve_info* info);
/* Preconditioner.apply(b, x) on host vectors (after rsg_solver_setup). */
rsg_status rsg_precond_apply(rsg_solver* s, const double* b, double* x);
/* Preconditioner.transApply(b, x) */
rsg_status rsg_precond_trans_apply(rsg_solver* s, const double* b, double* x);
/* Residual history of the last solve (monitor values in call order). */
rsg_status rsg_solver_history(rsg_solver* s, int32_t max_len, double* out, int32_t* len);
/* AMG hierarchy built by rsg_solver_setup (sparse/AMG.java:224-286), for
 * inspection: the number of levels, and per level k its operator (CSR), the
 * aggregate of each node (pt, -1 if none) and the smoothed interpolation in
 * CompColMatrix form (colptr, rowind, data).  sizes = {n, nnz, coarse size,
 * nnz of the interpolation}; the coarse size is 0 on the last level.  Any
 * array may be NULL.  No counterpart in the reference (its fields are private). */
rsg_status rsg_solver_amg_levels(rsg_solver* s, int32_t* levels);
rsg_status rsg_solver_amg_level(rsg_solver* s, int32_t k, int32_t* sizes, int32_t* rowptr, int32_t* col,
                                double* val, int32_t* pt, int32_t* colptr, int32_t* rowind, double* idata);

/* No-allocation CG: conjugate gradients with the diagonal preconditioner on
 * a CSR matrix and vectors that are already in device memory, for callers
 * that cannot allocate device memory while they run (a host runtime that
 * has reserved the GPU memory it may use, or a loop that forbids
 * allocation).  No counterpart in the reference: it computes what
 * rsg_solver_solve computes for RSG_CG with RSG_PC_DIAGONAL, with the same
 * reduction order.
 *
 * All workspace (five vectors of n doubles plus reduction partials, about
 * 40 MiB) is one static device array.  The driver reserves it on a device
 * when it loads the library's module there (with CUDA's default lazy module
 * loading: during the first call on that device) and the device holds it
 * until the process exits; a caller whose device memory is spoken for after
 * start-up makes one call with a 1-row system at start-up, or runs with
 * CUDA_MODULE_LOADING=EAGER.  n may not exceed RSG_NOALLOC_MAX_ROWS
 * (RSG_BAD_ARG otherwise).  The entry point calls no cudaMalloc or cudaFree.
 * Its first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture
 * begins.  After cudaDeviceReset on a device the looked-up address is
 * stale: do not call the entry point on that device again in the process.
 * Every call shares the array: calls that overlap on the GPU (different
 * streams or threads) race and must be serialised by the caller.  A zero
 * diagonal returns RSG_ZERO_PIVOT whatever the residual, as
 * DiagonalPreconditioner.setMatrix fails before any iteration.
 * stream: a cudaStream_t, or NULL for the default stream.  The call returns
 * when the solve has finished; d_x holds the result (also on failure). */
#define RSG_NOALLOC_MAX_ROWS 1048576
rsg_status rsg_cg_diagonal_noalloc(int32_t device, void* stream, int32_t n, int32_t nnz, const int32_t* d_row_ptr,
                                   const int32_t* d_col, const double* d_val, const double* d_b, double* d_x,
                                   double rtol, double atol, double dtol, int32_t max_iter, rsg_solve_info* info);

/* ------------------------------------------------- mesh + MPFA-O -------- */
/* Structured hexahedral (dim 3) or quadrilateral (dim 2, nk = 0) mesh in
 * RS's StructuredMeshGenerator numbering.  coords: 3 doubles per corner point
 * in linear point order (i fastest), or NULL for the tensor grid built from
 * (x0, y0, z0) and spacings (dx, dy, dz), dz < 0 as RS requires.
 * perm: 6 doubles per element (xx, yy, zz, xy, xz, yz), RockDataParser's
 * permx..permyz. */
rsg_status rsg_mesh_create_structured(rsg_ctx* ctx, int32_t dim, int32_t ni, int32_t nj, int32_t nk,
                                      const double* coords, double x0, double y0, double z0, double dx, double dy,
                                      double dz, const double* perm, rsg_mesh** out);
rsg_status rsg_mesh_destroy(rsg_mesh* m);
/* O_MPFA.calculateTransmissibilities + Connection.setDarcyTransmissibilities,
 * on the GPU.  continuity in (0, 1] (O_MPFA "Continuity" key). */
rsg_status rsg_mesh_compute_mpfa(rsg_mesh* m, double continuity);
/* TPFA.calculateTransmissibilities (geometry/flux/TPFA.java:31-72), the
 * reference's two-point alternative, on the GPU: two MD entries per
 * connection, (here, t) and (there, -t), with TPFA's distance weighting. */
rsg_status rsg_mesh_compute_tpfa(rsg_mesh* m);
/* L_MPFA.calculateTransmissibilities (geometry/flux/L_MPFA.java:52-74), the
 * L-method, on the GPU (3-D meshes; RSG_UNSUPPORTED in 2-D): at every
 * interior corner point each connection takes the L interaction region (its
 * here or there element and that element's three face neighbours at the
 * point) whose primary coefficient is smaller in magnitude; boundary points
 * take a two-point flux over the sub-face.  The reference orders a list's
 * entries through hash sets; here they follow the corner points in
 * ascending order, a region's elements primary first.  The discrete adjoint
 * (rsg_mesh_transmissibility_adjoint, rsg_sim_backward) is not built for
 * L-method lists and returns RSG_UNSUPPORTED. */
rsg_status rsg_mesh_compute_lmpfa(rsg_mesh* m);
/* counts[0] elements, [1] connections, [2] MD entries, [3] corner points,
 * [4] pressure-pattern nnz (valid after MPFA) */
rsg_status rsg_mesh_get_counts(rsg_mesh* m, int64_t* counts);
/* centers: 3 per element; volumes: 1 per element (either may be NULL) */
rsg_status rsg_mesh_get_geometry(rsg_mesh* m, double* centers, double* volumes);
/* conn: 2 per connection (here, there) */
rsg_status rsg_mesh_get_connections(rsg_mesh* m, int32_t* conn);
/* MD lists: md_ptr (connections+1), md_elem and md_k (MD entries) */
rsg_status rsg_mesh_get_transmissibilities(rsg_mesh* m, int32_t* md_ptr, int32_t* md_elem, double* md_k);
/* which = 0: LinearSolver pattern (with diagonal); 1: PotentialCalculator
 * pattern (without the explicit diagonal).  row_ptr: elements+1, col: nnz
 * (query nnz first with col == NULL). */
rsg_status rsg_mesh_get_pattern(rsg_mesh* m, int32_t which, int32_t* row_ptr, int32_t* col, int64_t* nnz);
/* PotentialCalculator.discretizeFlux into a CSR created with pattern 1:
 * A(here,k) += t_k, A(there,k) -= t_k (numerics/PotentialCalculator.java:319-333). */
rsg_status rsg_mesh_assemble_potential(rsg_mesh* m, rsg_csr* A);
/* Connection fluxes: flux[c] = sum over c's MD list of t_k p[element_k], in
 * list order (PotentialCalculator.calculateFlux, numerics/
 * PotentialCalculator.java:265-280; LocalFlowRateAverage.computeDarcyFlux,
 * upscale/LocalFlowRateAverage.java:123-137).  p: elements doubles, flux:
 * connections doubles (host).  Valid after MPFA or TPFA. */
rsg_status rsg_mesh_connection_flux(rsg_mesh* m, const double* p, double* flux);
/* Centre of each connection's here interface (Connection.hereInterface()
 * .center, which meshgen/partition/PartitionData.java:318,365 classifies):
 * 3 doubles per connection (host). */
rsg_status rsg_mesh_get_interface_centers(rsg_mesh* m, double* centers);

/* ------------------------------------------------------- upscaling ----- */
/* upscale/PressureDiscretisation(mesh, bc) (upscale/PressureDiscretisation
 * .java:59-196): the steady single-phase pressure problem of flow-based
 * upscaling.  Pattern without the explicit diagonal; A(here,k) += t_k,
 * A(there,k) -= t_k over every connection; for each of the nbc boundary
 * cells b_i = values[q] and row i := e_i (Matrices.zeroRows(A, 1.0, {i})),
 * every other b_i = 0 (a cell listed twice keeps its last value).  Solved on
 * the GPU by GMRES(30) + ILU(0) from x = 0 with the reference's
 * DefaultIterationMonitor (10000 iterations, rtol 1e-50, atol 1e-10, dtol
 * 1e5).  x: elements doubles out (host), also on failure; info (may be NULL)
 * the solve.  Returns the solve's status (RSG_NOT_CONVERGED_* as
 * IterativeSolverNotConvergedException's reasons). */
rsg_status rsg_upscale_pressure(rsg_mesh* m, int32_t nbc, const int32_t* cells, const double* values, double* x,
                                rsg_solve_info* info);

/* ------------------------------------------------ discrete adjoint ------ */
/* No reference counterpart: reverse-mode derivatives of the MPFA-O
 * transmissibilities (T = C A^-1 B - D of O_MPFA.java:193-239) with respect
 * to the natural logarithm of each element's permeability tensor (K_e scaled
 * by exp(theta_e)).  For npairs pairs of connection weights mu_k
 * (npairs x connections) and element potentials phi_k (npairs x elements),
 *   dlogk[e] = sum_k sum_c mu_k[c] d(sum_m t_cm phi_k[el_m]) / d theta_e.
 * Valid after rsg_mesh_compute_mpfa; host arrays. */
rsg_status rsg_mesh_transmissibility_adjoint(rsg_mesh* m, int32_t npairs, const double* conn_weights,
                                             const double* cell_potentials, double* dlogk);
/* Discrete adjoint of the steady potential problem of PotentialCalculator
 * (numerics/PotentialCalculator.java:319-333): A(theta) p = b with A
 * assembled by rsg_mesh_assemble_potential and the nfixed rows in fixed
 * replaced by identity rows (rsg_csr_zero_rows with diagonal 1), p its
 * solution.  For J(p) with gradient dJdp, solves A^T lambda = dJdp with the
 * given solver (its preconditioner and monitor), then
 *   dJ/dtheta_e = -sum_c (lambda~_here - lambda~_there) dF_c/dtheta_e,
 * lambda~ being lambda with the fixed rows zeroed and F_c = sum_m t_cm p_m
 * the connection flux.  lambda (may be NULL) receives the adjoint solution,
 * dJ_dlogk the gradient; info the transposed solve.  The solver is set up on
 * A^T inside the call and left without a matrix: call rsg_solver_setup again
 * before its next solve. */
rsg_status rsg_potential_adjoint(rsg_mesh* m, rsg_solver* solver, rsg_csr* A, int32_t nfixed, const int32_t* fixed,
                                 const double* p, const double* dJdp, double* lambda, double* dJ_dlogk,
                                 rsg_solve_info* info);

/* -------------------------------------------- fluid / rock / sources --- */
enum { RSG_FN_CONSTANT = 0, RSG_FN_TABLE = 1, RSG_FN_EVEN_TABLE = 2 };
/* util/Function: ConstantValue, LookupTable (1-3D) or EvenLookupTable. */
typedef struct {
  int32_t kind;
  int32_t dim;          /* number of arguments */
  double value;         /* RSG_FN_CONSTANT */
  int32_t n[3];         /* table points per axis */
  const double* coord[3]; /* TABLE: n[d] sorted coordinates; EVEN: {min, max} */
  const double* data;   /* n0*n1*n2 values, axis 0 fastest (LookupTable "data") */
} rsg_function;

/* BlackOilEquationOfState (fluid/BlackOilEquationOfState.java) on top of
 * WaterEquationOfState (fluid/WaterEquationOfState.java).  Component 0 is
 * water (fluid/Components.java:56-65). */
typedef struct {
  int32_t nc;
  double molecular_weight[RSG_MAX_COMPONENTS];
  int32_t group[RSG_MAX_COMPONENTS]; /* 0 water, 1 oil group, 2 gas group */
  rsg_function water_density, water_viscosity, water_enthalpy; /* f(p, T) */
  rsg_function bubble_point, dew_point;                        /* f(p, T) */
  rsg_function oil_density, gas_density, oil_viscosity, gas_viscosity; /* f(p, C, T) */
  rsg_function oil_enthalpy, gas_enthalpy;
} rsg_blackoil;

/* CoreyRockFluid (rock/CoreyRockFluid.java:41-82), phases water, oil, gas */
typedef struct {
  double Sr[3], n[3], ke[3];
  double cw, cow, cg, cog, aw, aow, ag, aog;
} rsg_corey;

enum { RSG_SOURCE_FIXED = 0, RSG_SOURCE_REGULAR = 1 };
/* Tabular rock-fluid models in place of Corey (rsg_sim_set_rock_tables):
 * RSG_RF_TABULAR is rock/TabularRockFluid.java:31-93: 1D tables krw(Sw),
 * krg(Sg), krow(So), krog(So + Sw), kro = (Sg krog(So + Sw) + Sw krow(So)) /
 * (Sg + Sw) (water must be present), pcow(Sw), pcgo(Sg);
 * RSG_RF_THREE_PHASE_TABULAR is rock/ThreePhaseTabularRockFluid.java:31-80:
 * 2D tables krw, krg, kro, pcow, pcgo of (Sw, Sg).  Relative permeability
 * tables must stay within [0, 1]; capillary pressures default to the
 * constant 0 (kind RSG_FN_CONSTANT, value 0). */
enum { RSG_RF_COREY = 0, RSG_RF_TABULAR = 1, RSG_RF_THREE_PHASE_TABULAR = 2 };
typedef struct {
  int32_t kind;
  rsg_function krw, krg, krow, krog, kro, pcow, pcgo;
} rsg_rock_tables;

/* field/Source.java: Fixed (locked cells) and Regular (mol/s per element) */
typedef struct {
  int32_t type;
  int32_t num_elements;
  const int32_t* elements;
  double q[RSG_MAX_COMPONENTS];
  double temperature;
  double fraction[RSG_MAX_COMPONENTS];
} rsg_source;

/* field/InitialValues.java */
typedef struct {
  double datum_depth;
  double datum_pressure;
  rsg_function temperature;                     /* f(z) */
  rsg_function fraction[RSG_MAX_COMPONENTS];   /* f(z) */
} rsg_initial;

/* numerics/RunSpec.java:133-251 (names kept) */
typedef struct {
  int32_t max_nonlinear_pressure_iterations; /* 10 */
  double pressure_tolerance;                 /* 1e-6 */
  int32_t linear_solver;                     /* RSG_BICGSTAB */
  int32_t preconditioner;                    /* RSG_PC_ILU */
  int32_t max_linear_iterations;             /* 5000 */
  double relative_tolerance;                 /* 1e-50 */
  double absolute_tolerance;                 /* 1e-12 */
  double divergence_tolerance;               /* 1e5 */
  int32_t truncate_negative_moles;           /* 0 */
  int32_t newton_stop_rule;  /* 0: RS rule dp[0] < tol (Discretisation.java:324); 1: max |dp/p| < tol */
  double omega, ax, ay;      /* BodyForces (field/Field.java:184-202) */
  int32_t gmres_restart;     /* 30 */
  /* RSG_FGMRES_MIXED only (no RunSpec counterpart): FP32 inner BiCGstab steps
   * per outer step and the inner relative tolerance; 0 keeps 10 and 1e-3 */
  int32_t inner_iterations;
  double inner_tolerance;
} rsg_runspec;

typedef struct {
  int32_t newton_iterations;
  int32_t linear_iterations;   /* summed over the Newton iterations */
  double dp_max;               /* last max |dp/p| */
  double dp0;                  /* last correction of element 0 */
  double mass_balance_error;   /* max over components, relative */
  int32_t status;
} rsg_step_info;

/* Field construction + initialisation by local volume balance, on the GPU. */
rsg_status rsg_sim_create(rsg_ctx* ctx, rsg_mesh* m, const rsg_blackoil* fluid, const rsg_corey* rockfluid,
                          const double* porosity, const double* compaction, int32_t nsources,
                          const rsg_source* sources, const rsg_initial* init, const rsg_runspec* spec,
                          rsg_sim** out);
rsg_status rsg_sim_destroy(rsg_sim* s);
/* Discretisation.solve(dt): pressure Newton loop, explicit molar masses,
 * secondaries.  On failure the state is left as the reference leaves it;
 * rsg_sim_retract restores the state stored at the start of the step
 * (Field.retract). */
rsg_status rsg_sim_step(rsg_sim* s, double dt, rsg_step_info* info);
rsg_status rsg_sim_retract(rsg_sim* s);
/* A device-side copy of the whole simulator state: time, pressures,
 * temperatures, moles, and the per-phase records and presence flags the next
 * step reads.  rsg_sim_save_state keeps one copy per simulator (replacing the
 * previous one); rsg_sim_restore_state returns to it, after which the same
 * steps repeat bit for bit (RSG_BAD_ARG if nothing was saved).  Like
 * Field.retract (field/Field.java:535-545), which returns one step, but to
 * any saved point; RS keeps such points as serialised Field objects
 * (numerics/Main.java:86-105). */
rsg_status rsg_sim_save_state(rsg_sim* s);
rsg_status rsg_sim_restore_state(rsg_sim* s);
/* Replaces the simulator's rock-fluid model (RockFluid.create's "Tabular" and
 * "ThreePhaseTabular" choices) and recomputes the secondaries.  RSG_RF_COREY
 * returns to the Corey model the simulator was created with.  Table
 * arrays are copied.  RSG_BAD_ARG for wrong table dimensions or relative
 * permeabilities outside [0, 1]. */
rsg_status rsg_sim_set_rock_tables(rsg_sim* s, const rsg_rock_tables* t);
/* Restart files (numerics/Main.java:86-105 saves the Field at report times;
 * field/Field.java:207-262 restarts from its primary variables).  The file
 * holds time, p, reference pressure, T and N: "RSGRST01", int32 n, nc, 1, 0,
 * float64 time, then float64 p[n], p0[n], T[n], N[nc][n].
 * rsg_sim_read_restart needs a simulator of the same n and nc (RSG_BAD_ARG
 * otherwise), loads the primaries, drops the per-phase records of earlier
 * evaluations as new control volumes would, and recomputes the secondaries.
 * Fixed source cells keep the values in the file (Field's constructor
 * re-balances them, which returns the same values while their pressure,
 * temperature and composition are those of the run that wrote the file). */
rsg_status rsg_sim_write_restart(rsg_sim* s, const char* path);
rsg_status rsg_sim_read_restart(rsg_sim* s, const char* path);
/* Discrete adjoint of a simulator run (Discretisation's sequential pressure
 * Newton step and explicit molar update, numerics/Discretisation.java:280-919;
 * black-oil fluids with at most 3 components).  rsg_sim_forward runs nsteps
 * steps of sizes dt[] from the current state, keeping a state checkpoint
 * every checkpoint_every steps, and accumulates the objective
 *   J = sum over steps, over the ncells listed cells and the components of
 *       cell_weights[j] * component_weights[nu] * dN
 * (dN: the step's molar change of that cell before locking, so for a Fixed
 * (locked) producer cell the moles produced into it).  rsg_sim_backward then
 * sweeps the steps in reverse, recomputing each block of steps from its
 * checkpoint, solving the transposed exact pressure Jacobian per step with
 * the simulator's Krylov method and preconditioner to relative tolerance
 * rtol, and returns dJ/dlog k per element (through the MPFA-O
 * transmissibilities), optionally dJ/dp and dJ/dN of the initial state.  The
 * Newton iterations of the forward run are taken as converged (F = 0).  The
 * simulator is left at the end state of the forward run. */
typedef struct {
  int32_t steps;                     /* forward steps */
  int32_t newton_iterations;         /* forward Newton iterations */
  int32_t linear_iterations;         /* forward linear iterations */
  int32_t recomputed_steps;          /* steps re-run from checkpoints */
  int32_t backward_steps;
  int32_t adjoint_linear_iterations; /* iterations of the transposed solves */
  double objective;                  /* J of the forward run */
} rsg_adjoint_info;
rsg_status rsg_sim_forward(rsg_sim* s, int32_t nsteps, const double* dt, int32_t checkpoint_every, int32_t ncells,
                           const int32_t* cells, const double* cell_weights, const double* component_weights,
                           double* objective, rsg_adjoint_info* info);
rsg_status rsg_sim_backward(rsg_sim* s, double rtol, double* dJ_dlogk, double* dJ_dp0, double* dJ_dN0,
                            rsg_adjoint_info* info);
/* p: n; N: nc*n (component major); S: 3*n (phase major) — any may be NULL */
rsg_status rsg_sim_get_state(rsg_sim* s, double* p, double* N, double* S);
rsg_status rsg_sim_set_state(rsg_sim* s, const double* p, const double* N);
/* Last assembled pressure Jacobian (values in the pressure pattern order)
 * and right-hand side, before the locked-row treatment. */
rsg_status rsg_sim_get_jacobian(rsg_sim* s, double* values, double* rhs);
/* Per-cell secondaries after the last update: R, dRdp (n each). */
rsg_status rsg_sim_get_residual_volume(rsg_sim* s, double* R, double* dRdp);

/* Time-step control: the RunSpec keys of numerics/RunSpec.java:146-204 (the
 * defaults are those of RunSpec). */
typedef struct {
  double lambda;                        /* Lambda, 0.5 */
  double target_residual_volume;        /* TargetResidualVolume, 1e-2 */
  int32_t target_nonlinear_iterations;  /* TargetNonLinearPressureIterations, 5 */
  double target_throughput;             /* TargetThroughputRatio, 0.5 */
  double dt_min, dt_max;                /* TimeStepMinimum, TimeStepMaximum [s] */
} rsg_dt_control;

typedef struct {
  double residual_volume, pressure_iterations, throughput; /* the three dt factors */
  int32_t limit; /* 0 none, 1 maximum timestep, 2 residual volume, 3 pressure iterations, 4 throughput */
} rsg_dt_factors;

typedef struct {
  int32_t steps, retries;           /* accepted steps, retracted attempts */
  int32_t newton_iterations, linear_iterations;
  double time;                      /* field time reached [s] */
  int32_t status;                   /* status of the last attempt */
} rsg_step_to_info;

/* ------------------------------------------- cubic equation of state --- */
/* fluid/CubicEquationOfState.java: Peng-Robinson (or Soave-Redlich-Kwong)
 * hydrocarbon phases with an isothermal flash, plus the water phase of
 * WaterEquationOfState.  Component 0 is water; 1..nc-1 are hydrocarbons.
 * Units are SI (K, Pa, kg/mol, m3/mol). */
enum { RSG_EOS_PR = 0, RSG_EOS_SRK = 1 };
typedef struct {
  int32_t nc;                                   /* components including water */
  int32_t eos;                                  /* RSG_EOS_PR (EOS key "PR") */
  double Tc[RSG_MAX_COMPONENTS], pc[RSG_MAX_COMPONENTS], omega[RSG_MAX_COMPONENTS];
  double Mw[RSG_MAX_COMPONENTS], Vc[RSG_MAX_COMPONENTS];
  double shift[RSG_MAX_COMPONENTS];             /* volume shift s (ComponentData/<name>/s) */
  double bic[RSG_MAX_COMPONENTS * RSG_MAX_COMPONENTS]; /* binary interaction dij, row major, symmetric */
  double flash_criteria;                        /* FlashSwitchingCriteria: SS above, NR below (1e4) */
  double flash_tolerance;                       /* FlashTolerance on max |f_oil - f_gas| [Pa] (1e-1) */
  int32_t flash_max_iterations;                 /* no counterpart (the Java loop is unbounded) */
  double lbc[5];                                /* Viscosity a1..a5 (0.1023, 0.023364, 0.058533, -0.040758, 0.0093324) */
  rsg_function water_density, water_viscosity;  /* f(p, T) */
} rsg_cubic_fluid;

/* Per-phase record of EquationOfStateData, as doubles per cell:
 * field f of phase a (0 water, 1 oil, 2 gas) of cell i lives at
 * phases[(a * RSG_CUBIC_FIELDS(nc) + f) * n + i]; fields: present (0/1), V,
 * xi, dVdp, dVdT, mu, N[nc], dVdN[nc]. */
#define RSG_CUBIC_FIELDS(nc) (6 + 2 * (nc))
/* CubicEquationOfState.calculatePhaseState for n cells (p, T: n; N: nc x n,
 * component major).  phases is in/out: the oil and gas compositions it holds
 * start the flash where both phases were present, as the Java object's
 * persisted phase data do.  iterations (n, may be NULL) receives the flash
 * iterations per cell.  Host arrays, one thread per cell on the GPU. */
rsg_status rsg_cubic_phase_state(rsg_ctx* ctx, const rsg_cubic_fluid* fluid, int32_t n, const double* p,
                                 const double* T, const double* N, double* phases, int32_t* iterations);
/* The same, with a status per cell (cell_status: n, 0 = OK, else the
 * rsg_status of that cell's failure); every cell is evaluated and the call
 * returns RSG_OK unless the arguments or the GPU fail. */
rsg_status rsg_cubic_phase_state_cells(rsg_ctx* ctx, const rsg_cubic_fluid* fluid, int32_t n, const double* p,
                                       const double* T, const double* N, double* phases, int32_t* iterations,
                                       int32_t* cell_status);

/* rsg_sim_create with the cubic equation of state as the fluid model
 * (compositional runs): CV.calculateFluidProperties calls
 * CubicEquationOfState.calculatePhaseState for every cell. */
rsg_status rsg_sim_create_cubic(rsg_ctx* ctx, rsg_mesh* mesh, const rsg_cubic_fluid* fluid, const rsg_corey* rf,
                                const double* porosity, const double* compaction, int32_t nsources,
                                const rsg_source* sources, const rsg_initial* init, const rsg_runspec* spec,
                                rsg_sim** out);

/* Ensembles: rsg_sim_step on every member, concurrently.  Each member must
 * own its context (its own stream); members are driven from up to
 * max_concurrent host threads (0: one per member), so their kernels overlap
 * on the GPU.  Returns the first failing member's status (statuses[i] and
 * infos[i] hold each member's).  Results equal stepping each member alone.
 * No counterpart in the reference (RS runs one field per process). */
rsg_status rsg_ensemble_step(int32_t count, rsg_sim* const* sims, const double* dt, int32_t max_concurrent,
                             rsg_step_info* infos, int32_t* statuses);
/* Ensembles in lockstep: one time step of dt[i] on every member, with the
 * pressure solves of all members in ONE persistent launch per Newton
 * iteration.  Each member's Discretisation.solve(dt)
 * (numerics/Discretisation.java:208-225) runs as in rsg_sim_step: the
 * members assemble their Jacobians and factor their ILU(0) preconditioners on
 * their own streams, then one kernel of thread-block clusters takes the
 * members from a work queue and solves each pressure system completely
 * (BiCGstab, mtj/.../sparse/BiCGstab.java:65-116, with ILU(0)) through
 * per-member offsets, and each member updates its pressure and tests its
 * Newton convergence; converged members leave the loop.  Members must use
 * RSG_BICGSTAB with RSG_PC_ILU.  precision 0: BiCGstab in FP64 with the
 * FP64 ILU(0) factors; 1: the mixed-precision solver of RSG_FGMRES_MIXED
 * (FP64 flexible GMRES with the solver's restart around its inner FP32
 * BiCGstab steps on the FP32 factors and the FP32 copy of A), so the
 * relative residual is met in FP64.  A member whose
 * step fails stops there (statuses[i], infos[i]); the others go on.  Returns
 * the first failing member's status.  Results agree with rsg_sim_step per
 * member to the Krylov solver's rounding (the dot products are summed in a
 * different order) and do not depend on the number of members or on their
 * order.  No counterpart in the reference (RS runs one field per process). */
rsg_status rsg_ensemble_step_batched(int32_t count, rsg_sim* const* sims, const double* dt, int32_t precision,
                                     rsg_step_info* infos, int32_t* statuses);
/* IterativeSolver.solve (mtj/.../sparse/IterativeSolver.java:43-74) on many
 * independent systems in ONE persistent launch: solvers[i] (RSG_BICGSTAB with
 * RSG_PC_ILU, set up with A[i] by rsg_solver_setup) solves A[i] x[i] = b[i]
 * from the initial guess x[i], host arrays as in rsg_solver_solve.  The
 * launch is the ensemble solver of rsg_ensemble_step_batched (precision as
 * there); statuses[i] and infos[i] report each system (MTJ's reasons;
 * RSG_UNSUPPORTED for another method or preconditioner; RSG_BAD_ARG for a
 * solver not set up with its matrix), x[i] is copied back either way, and
 * the first failing status is returned.  No counterpart in the reference. */
rsg_status rsg_solver_solve_batched(int32_t count, rsg_solver* const* solvers, rsg_csr* const* A,
                                    const double* const* b, double* const* x, int32_t precision,
                                    rsg_solve_info* infos, int32_t* statuses);
/* Matrix Market exchange files (mtj/src/no/uib/cipr/matrix/io/
 * MatrixVectorReader.java, MatrixVectorWriter.java).  Host code: paths are
 * files of the calling process.
 * rsg_mm_read_matrix_size + rsg_mm_read_csr: CompRowMatrix(MatrixVectorReader)
 * (sparse/CompRowMatrix.java:68-146): coordinate real/integer files, general,
 * symmetric (mirrored) or skew-symmetric (negated mirror), optional header,
 * '%' comments; rows sorted, a repeated entry keeps its last value; *nnz is
 * the number of stored entries after the mirroring.  Pattern, complex and
 * array matrices: RSG_UNSUPPORTED; unreadable or ill-formed files and indices
 * out of range: RSG_BAD_ARG.
 * rsg_mm_write_csr: MatrixVectorWriter's "%%MatrixMarket matrix coordinate
 * real general", "%10d %10d %19d" and "%10d %10d % .12e" lines, 1-based, in
 * CSR order.
 * rsg_mm_read_vector_size + rsg_mm_read_vector: DenseVector(MatrixVectorReader)
 * (DenseVector.java:52-96), array or coordinate.  rsg_mm_write_vector:
 * "%%MatrixMarket vector array real", "%10d", "% .12e" per entry. */
rsg_status rsg_mm_read_matrix_size(const char* path, int32_t* rows, int32_t* cols, int64_t* nnz);
rsg_status rsg_mm_read_csr(const char* path, int32_t rows, int64_t nnz, int32_t* row_ptr, int32_t* col, double* val);
rsg_status rsg_mm_write_csr(const char* path, int32_t rows, int32_t cols, const int32_t* row_ptr, const int32_t* col,
                            const double* val);
rsg_status rsg_mm_read_vector_size(const char* path, int32_t* size);
rsg_status rsg_mm_read_vector(const char* path, int32_t size, double* x);
rsg_status rsg_mm_write_vector(const char* path, int32_t size, const double* x);
/* Field.getTime: advanced by every rsg_sim_step, restored by rsg_sim_retract. */
rsg_status rsg_sim_get_time(rsg_sim* s, double* t);
/* Discretisation.calculateDt(dt) (numerics/Discretisation.java:928-1002): the
 * next time step after a successful step of size dt. */
rsg_status rsg_sim_calculate_dt(rsg_sim* s, double dt, const rsg_dt_control* c, double* dt_new, rsg_dt_factors* f);
/* Discretisation.throughputFactor (:986-998) */
rsg_status rsg_sim_throughput_factor(rsg_sim* s, const rsg_dt_control* c, double* factor);
/* TimeStepper.stepTo(endTime) (numerics/TimeStepper.java:58-102): steps to
 * end_time; a step that fails with a SolverFailure status (1, 2, 3, 7, 8, 13)
 * is retracted and retried with dt * min(1/2, throughputFactor) while
 * dt > dt_min.  *dt is the time step carried between calls (TimeStepper.dt,
 * dt_min initially). */
rsg_status rsg_sim_step_to(rsg_sim* s, double end_time, const rsg_dt_control* c, double* dt, rsg_step_to_info* info);

#ifdef __cplusplus
}
#endif
#endif /* RSG_H */
