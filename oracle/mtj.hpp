// Oracle (test infrastructure only): CPU restatement of the Matrix Toolkits
// for Java (MTJ) sparse stack used by RS.  Only tests/, the smoke check and
// bench.py's CPU-baseline leg may load this code; the product never does.
//
// Every routine follows one Java method line by line and cites it as
// mtj/src/no/uib/cipr/matrix/<file>:<lines>.  Arithmetic is plain IEEE
// double, evaluated in the Java source order (built with -ffp-contract=off so
// that no multiply-add is fused).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace orc {

// Failure classes crossing the oracle's C boundary.  The numbering is shared
// with the GPU library's rsg_status (include/rsg.h).
enum Status : int32_t {
  ST_OK = 0,
  ST_NOT_CONVERGED_ITERATIONS = 1,  // NotConvergedException.Reason.Iterations
  ST_NOT_CONVERGED_DIVERGENCE = 2,  // Reason.Divergence (includes NaN)
  ST_NOT_CONVERGED_BREAKDOWN = 3,   // Reason.Breakdown
  ST_ZERO_PIVOT = 4,                // ILU.factor RuntimeException
  ST_MISSING_DIAGONAL = 5,          // ILU.findDiagonalIndices RuntimeException
  ST_OUT_OF_PATTERN = 6,            // CompRowMatrix.getIndex IndexOutOfBounds
  ST_NONPOSITIVE_PRESSURE = 7,      // Discretisation.updatePressure
  ST_NEGATIVE_MOLES = 8,            // Discretisation.updateMolarMass
  ST_BAD_ARG = 9,
  ST_CUDA_ERROR = 10,
  ST_TIMEOUT = 11,
  ST_UNSUPPORTED = 12,
  ST_NEWTON_NOT_CONVERGED = 13,     // Discretisation.converged SolverFailure
  ST_SINGULAR = 14,                 // MatrixSingularException (dense LU)
  ST_PHYSICS = 15,                  // RuntimeException from CV / EOS checks
};

struct Failure : std::runtime_error {
  Status status;
  double residual;
  int iterations;
  Failure(Status s, const std::string& m, double r = 0, int it = 0)
      : std::runtime_error(m), status(s), residual(r), iterations(it) {}
};

using Vec = std::vector<double>;

// CompRowMatrix (mtj/src/no/uib/cipr/matrix/sparse/CompRowMatrix.java)
struct CompRowMatrix {
  int n = 0;
  std::vector<int> rowptr, col;
  Vec data;
  // construct(int[][] nz), CompRowMatrix.java:165-190: concatenate the rows
  // and sort the column indices within each row.
  static CompRowMatrix from_rows(int n, const std::vector<std::vector<int>>& nz);
  int nnz() const { return (int)col.size(); }
  int getIndex(int row, int column) const;          // :428-437
  void add(int row, int column, double v);          // :404-410
  void set(int row, int column, double v);          // :396-402
  double get(int row, int column) const;            // :412-423
  void zero();                                       // :449-453
  void mult(const Vec& x, Vec& y) const;             // :300-320
  void multAdd(double alpha, const Vec& x, Vec& y) const;  // :335-353
  void transMult(const Vec& x, Vec& y) const;        // :355-372
};

// Matrices.zeroRows (mtj/src/no/uib/cipr/matrix/Matrices.java:631-652)
void zeroRows(CompRowMatrix& A, double diagonal, const std::vector<int>& rows);

// DenseVector BLAS-1 (mtj/src/no/uib/cipr/matrix/DenseVector.java:190-295)
double dot(const Vec& a, const Vec& b);
double norm2(const Vec& a);
void vset(Vec& y, const Vec& x);                       // set(Vector)
void vset(Vec& y, double alpha, const Vec& x);         // set(double, Vector)
void vadd(Vec& y, const Vec& x);                       // add(Vector)
void vadd(Vec& y, double alpha, const Vec& x);         // add(double, Vector)
void vscale(Vec& y, double alpha);                     // scale(double)

// DefaultIterationMonitor (sparse/DefaultIterationMonitor.java:33-165) with
// the counters of AbstractIterationMonitor (:60-104).
struct IterationMonitor {
  int maxIter = 100000;
  double rtol = 1e-5, atol = 1e-50, dtol = 1e+5;
  int iter = 0;
  double initR = 0, residual = 0;
  std::vector<double>* history = nullptr;  // optional residual trace
  void setFirst() { iter = 0; }
  bool isFirst() const { return iter == 0; }
  void next() { iter++; }
  bool converged(double r);                 // :132-156
  bool converged(const Vec& r) { return converged(norm2(r)); }
};

struct Preconditioner {
  virtual ~Preconditioner() {}
  virtual void apply(const Vec& b, Vec& x) = 0;
  virtual void transApply(const Vec& b, Vec& x) = 0;
  virtual void setMatrix(const CompRowMatrix& A) = 0;
};

struct IdentityPreconditioner : Preconditioner {  // AbstractIterativeSolver.java:82-96
  void apply(const Vec& b, Vec& x) override { x = b; }
  void transApply(const Vec& b, Vec& x) override { x = b; }
  void setMatrix(const CompRowMatrix&) override {}
};

// DiagonalPreconditioner (sparse/DiagonalPreconditioner.java)
struct DiagonalPreconditioner : Preconditioner {
  Vec invdiag;
  void apply(const Vec& b, Vec& x) override;
  void transApply(const Vec& b, Vec& x) override { apply(b, x); }
  void setMatrix(const CompRowMatrix& A) override;
};

// ILU(0) (sparse/ILU.java:54-140) with the unit-lower and upper triangular
// solves of UnitLowerCompRowMatrix.java:48-86 and UpperCompRowMatrix.java:48-90.
struct ILU : Preconditioner {
  CompRowMatrix LU;
  std::vector<int> diagind;
  Vec y;
  void apply(const Vec& b, Vec& x) override;       // :64-70
  void transApply(const Vec& b, Vec& x) override;  // :72-78
  void setMatrix(const CompRowMatrix& A) override; // :80-84
  void factor();                                   // :86-125
};

// SSOR (sparse/SSOR.java) used as the AMG smoother and as a preconditioner.
struct SSOR : Preconditioner {
  CompRowMatrix F;
  std::vector<int> diagind;
  double omegaF = 1, omegaR = 1;
  bool reverse = true;
  Vec xx;
  void apply(const Vec& b, Vec& x) override;
  void transApply(const Vec& b, Vec& x) override { apply(b, x); }
  void setMatrix(const CompRowMatrix& A) override;
};

// Smoothed-aggregation AMG V-cycle (sparse/AMG.java) with the default
// parameters of AMG() (:204-206): SSOR(1, 1.85) pre- and SSOR(1.85, 1)
// post-smoothing, one of each, V-cycle, coarsest size 40, omega 2/3.
struct AMGLevel {
  CompRowMatrix A;              // Galerkin operator of this level
  std::vector<int> pt;          // tentative prolongation: aggregate of each node (-1: none)
  int c = 0;                    // coarse size
  std::vector<int> colptr, rowind;  // smoothed interpolation I (n x c), CompColMatrix
  Vec Idata;
  SSOR pre, post;
  Vec u, f, r;
};

struct AMG : Preconditioner {
  double omegaPreF = 1, omegaPreR = 1.85, omegaPostF = 1.85, omegaPostR = 1;
  int nu1 = 1, nu2 = 1, gamma = 1, min = 40;
  double omega = 2. / 3;
  std::vector<AMGLevel> L;  // L.size() == m; the last level keeps only A, u, f
  Vec lu;                   // LU factors of the coarsest operator (column major)
  std::vector<int> piv;
  int nc = 0;               // coarsest size
  bool singular = false;
  bool transpose = false;
  void apply(const Vec& b, Vec& x) override;       // AMG.java:208-214
  void transApply(const Vec& b, Vec& x) override;  // :216-222
  void setMatrix(const CompRowMatrix& A) override; // :224-286
  void cycle(int k);                               // :288-313
  void directSolve();                              // :315-323
};

enum Method : int32_t { M_CG = 0, M_BICGSTAB = 1, M_GMRES = 2 };
enum Precond : int32_t { P_NONE = 0, P_DIAGONAL = 1, P_ILU = 2, P_SSOR = 3, P_AMG = 4 };

// CG.solve (sparse/CG.java:58-87), BiCGstab.solve (sparse/BiCGstab.java:65-116),
// GMRES.solve (sparse/GMRES.java:127-176).  Each throws Failure on
// non-convergence exactly where the Java throws
// IterativeSolverNotConvergedException.
void cg_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& it);
void bicgstab_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& it);
void gmres_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& it, int restart);

// netlib dgetf2 (unblocked LU with partial pivoting, as dgetrf runs it for
// n below its block size) and dgetrs ('N' or 'T') on a column-major matrix.
int dgetf2(int n, double* A, int lda, int* ipiv);
void dgetrs(bool trans, int n, const double* A, int lda, const int* ipiv, double* b);

// Dense LU with partial pivoting as netlib LAPACK dgesv (dgetf2 + dgetrs),
// the routine MTJ's DenseMatrix.solve -> LUsolve reaches
// (mtj/src/no/uib/cipr/matrix/DenseMatrix.java:401,451-470).  A is n x n
// column-major, B is n x nrhs column-major and is overwritten with A\B.
// Returns 0, or j>0 if U(j,j) is exactly zero (LAPACK info).
int dgesv(int n, int nrhs, double* A, int lda, int* ipiv, double* B, int ldb);
// dgemm('N','N') with alpha = beta = 1: C += A*B (reference BLAS loop order).
void dgemm_nn_add(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc);
// dtrsm('L','U','N','N') on the leading n x n block: solves U x = b in place.
int dtrtrs_upper(int n, const double* A, int lda, double* b);

}  // namespace orc
