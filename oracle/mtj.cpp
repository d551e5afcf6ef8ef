// Oracle (test infrastructure only): restatement of MTJ's CompRowMatrix,
// DenseVector BLAS-1, iteration monitor, CG/BiCGstab/GMRES, ILU(0), SSOR,
// diagonal preconditioner and the netlib dense LU the MPFA code reaches.
#include "mtj.hpp"

#include <algorithm>
#include <cmath>

namespace orc {

// ---------------------------------------------------------------- CSR ----
CompRowMatrix CompRowMatrix::from_rows(int n, const std::vector<std::vector<int>>& nz) {
  // sparse/CompRowMatrix.java:165-190
  CompRowMatrix A;
  A.n = n;
  if ((int)nz.size() != n) throw Failure(ST_BAD_ARG, "nz.length != numRows");
  size_t nnz = 0;
  for (auto& r : nz) nnz += r.size();
  A.rowptr.assign(n + 1, 0);
  A.col.resize(nnz);
  A.data.assign(nnz, 0.0);
  for (int i = 1; i <= n; ++i) {
    A.rowptr[i] = A.rowptr[i - 1] + (int)nz[i - 1].size();
    for (int j = A.rowptr[i - 1], k = 0; j < A.rowptr[i]; ++j, ++k) {
      int c = nz[i - 1][k];
      if (c < 0 || c >= n) throw Failure(ST_BAD_ARG, "not a valid column index");
      A.col[j] = c;
    }
    std::sort(A.col.begin() + A.rowptr[i - 1], A.col.begin() + A.rowptr[i]);
  }
  return A;
}

// no.uib.cipr.matrix.sparse.Arrays.binarySearch: index of the key, or -1.
static int bsearch_row(const std::vector<int>& col, int key, int begin, int end) {
  int lo = begin, hi = end - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    if (col[mid] < key) lo = mid + 1;
    else if (col[mid] > key) hi = mid - 1;
    else return mid;
  }
  return -1;
}

int CompRowMatrix::getIndex(int row, int column) const {
  // CompRowMatrix.java:428-437
  int i = bsearch_row(col, column, rowptr[row], rowptr[row + 1]);
  if (i != -1 && col[i] == column) return i;
  throw Failure(ST_OUT_OF_PATTERN, "Entry (" + std::to_string(row + 1) + ", " +
                                       std::to_string(column + 1) + ") is not in the matrix structure");
}

void CompRowMatrix::add(int row, int column, double v) { data[getIndex(row, column)] += v; }
void CompRowMatrix::set(int row, int column, double v) { data[getIndex(row, column)] = v; }
double CompRowMatrix::get(int row, int column) const {
  int i = bsearch_row(col, column, rowptr[row], rowptr[row + 1]);
  return i >= 0 ? data[i] : 0.0;
}
void CompRowMatrix::zero() { std::fill(data.begin(), data.end(), 0.0); }

void CompRowMatrix::mult(const Vec& x, Vec& y) const {
  // CompRowMatrix.java:300-320 (DenseVector branch): y is zeroed and only
  // rows whose dot product is non-zero are written.
  std::fill(y.begin(), y.end(), 0.0);
  for (int i = 0; i < n; ++i) {
    double d = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; j++) d += data[j] * x[col[j]];
    if (d != 0) y[i] = d;
  }
}

void CompRowMatrix::multAdd(double alpha, const Vec& x, Vec& y) const {
  // CompRowMatrix.java:335-353
  for (int i = 0; i < n; ++i) {
    double d = 0;
    for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) d += data[j] * x[col[j]];
    y[i] += alpha * d;
  }
}

void CompRowMatrix::transMult(const Vec& x, Vec& y) const {
  // CompRowMatrix.java:355-372
  std::fill(y.begin(), y.end(), 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = rowptr[i]; j < rowptr[i + 1]; ++j) y[col[j]] += data[j] * x[i];
}

void zeroRows(CompRowMatrix& A, double diagonal, const std::vector<int>& rows) {
  // Matrices.java:631-652: every stored entry of a selected row becomes 0,
  // the diagonal becomes `diagonal` (and must exist in the pattern).
  std::vector<int> rs(rows);
  std::sort(rs.begin(), rs.end());
  for (int r : rs) {
    for (int j = A.rowptr[r]; j < A.rowptr[r + 1]; ++j)
      A.data[j] = (A.col[j] == r) ? diagonal : 0.0;
  }
  if (diagonal != 0)
    for (int r : rows) A.set(r, r, diagonal);
}

// ------------------------------------------------------------- BLAS-1 ----
double dot(const Vec& a, const Vec& b) {
  double d = 0.;
  for (size_t i = 0; i < a.size(); ++i) d += a[i] * b[i];
  return d;
}
double norm2(const Vec& a) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * a[i];
  return std::sqrt(s);
}
void vset(Vec& y, const Vec& x) { std::copy(x.begin(), x.end(), y.begin()); }
void vset(Vec& y, double alpha, const Vec& x) {
  if (alpha == 0) { std::fill(y.begin(), y.end(), 0.0); return; }
  for (size_t i = 0; i < y.size(); ++i) y[i] = alpha * x[i];
}
void vadd(Vec& y, const Vec& x) {
  for (size_t i = 0; i < y.size(); i++) y[i] += x[i];
}
void vadd(Vec& y, double alpha, const Vec& x) {
  if (alpha == 0) return;
  for (size_t i = 0; i < y.size(); i++) y[i] += alpha * x[i];
}
void vscale(Vec& y, double alpha) {
  for (size_t i = 0; i < y.size(); ++i) y[i] *= alpha;
}

// ------------------------------------------------------------ monitor ----
bool IterationMonitor::converged(double r) {
  // AbstractIterationMonitor.java:81-86 then DefaultIterationMonitor.java:132-156
  residual = r;
  if (history) history->push_back(r);
  if (isFirst()) initR = r;
  if (r < std::max(rtol * initR, atol)) return true;
  if (r > dtol * initR) throw Failure(ST_NOT_CONVERGED_DIVERGENCE, "Divergence", r, iter);
  if (iter >= maxIter) throw Failure(ST_NOT_CONVERGED_ITERATIONS, "Iterations", r, iter);
  if (std::isnan(r)) throw Failure(ST_NOT_CONVERGED_DIVERGENCE, "Divergence (NaN)", r, iter);
  return false;
}

// ----------------------------------------------------- preconditioners ----
void DiagonalPreconditioner::setMatrix(const CompRowMatrix& A) {
  // DiagonalPreconditioner.java:66-77
  invdiag.assign(A.n, 0.0);
  for (int i = 0; i < A.n; ++i) {
    double d = A.get(i, i);
    if (d == 0) throw Failure(ST_ZERO_PIVOT, "Zero diagonal on row " + std::to_string(i + 1));
    invdiag[i] = 1 / d;
  }
}
void DiagonalPreconditioner::apply(const Vec& b, Vec& x) {
  for (size_t i = 0; i < invdiag.size(); ++i) x[i] = b[i] * invdiag[i];
}

static std::vector<int> findDiagonalIndices(const CompRowMatrix& A) {
  // ILU.java:127-140
  std::vector<int> d(A.n);
  for (int k = 0; k < A.n; ++k) {
    d[k] = bsearch_row(A.col, k, A.rowptr[k], A.rowptr[k + 1]);
    if (d[k] < 0) throw Failure(ST_MISSING_DIAGONAL, "Missing diagonal entry on row " + std::to_string(k + 1));
  }
  return d;
}

void ILU::setMatrix(const CompRowMatrix& A) {
  // ILU.java:80-84: LU.set(A) copies values and structure, then factor().
  LU = A;
  y.assign(A.n, 0.0);
  factor();
}

void ILU::factor() {
  // ILU.java:86-125.  The inner scan of row k compares colind[l] before it
  // checks l against the row end, so when the scan runs off row k it reads
  // (and may update) the first entry of row k+1; that is reproduced here.
  const int n = LU.n;
  const int nnz = LU.nnz();
  auto& colind = LU.col;
  auto& rowptr = LU.rowptr;
  auto& data = LU.data;
  diagind = findDiagonalIndices(LU);
  for (int k = 1; k < n; ++k)
    for (int i = rowptr[k]; i < diagind[k]; ++i) {
      int index = colind[i];
      double LUii = data[diagind[index]];
      if (LUii == 0) throw Failure(ST_ZERO_PIVOT, "Zero pivot encountered on row " + std::to_string(i + 1));
      double LUki = (data[i] /= LUii);
      for (int j = diagind[index] + 1, l = rowptr[k] + 1; j < rowptr[index + 1]; ++j) {
        while (l < rowptr[k + 1] && colind[l] < colind[j]) l++;
        if (l >= nnz) throw Failure(ST_UNSUPPORTED, "ILU scan ran past the last row");
        if (colind[l] == colind[j]) data[l] -= LUki * data[j];
      }
    }
}

void ILU::apply(const Vec& b, Vec& x) {
  // L.solve(b, y): UnitLowerCompRowMatrix.java:48-67
  const int n = LU.n;
  for (int i = 0; i < n; ++i) {
    double sum = 0;
    for (int j = LU.rowptr[i]; j < diagind[i]; ++j) sum += LU.data[j] * y[LU.col[j]];
    // Java reads y (the output) for already finished rows.
    y[i] = b[i] - sum;
  }
  // U.solve(y, x): UpperCompRowMatrix.java:48-67
  for (int i = n - 1; i >= 0; --i) {
    double sum = 0;
    for (int j = diagind[i] + 1; j < LU.rowptr[i + 1]; ++j) sum += LU.data[j] * x[LU.col[j]];
    x[i] = (y[i] - sum) / LU.data[diagind[i]];
  }
}

void ILU::transApply(const Vec& b, Vec& x) {
  // U.transSolve(b, y): UpperCompRowMatrix.java:69-90
  const int n = LU.n;
  y = b;
  for (int i = 0; i < n; ++i) {
    y[i] /= LU.data[diagind[i]];
    for (int j = diagind[i] + 1; j < LU.rowptr[i + 1]; ++j) y[LU.col[j]] -= LU.data[j] * y[i];
  }
  // L.transSolve(y, x): UnitLowerCompRowMatrix.java:69-86
  x = y;
  for (int i = n - 1; i >= 0; --i)
    for (int j = LU.rowptr[i]; j < diagind[i]; ++j) x[LU.col[j]] -= LU.data[j] * x[i];
}

void SSOR::setMatrix(const CompRowMatrix& A) {
  // SSOR.java:126-141
  F = A;
  diagind.assign(A.n, 0);
  xx.assign(A.n, 0.0);
  for (int k = 0; k < A.n; ++k) {
    diagind[k] = bsearch_row(F.col, k, F.rowptr[k], F.rowptr[k + 1]);
    if (diagind[k] < 0) throw Failure(ST_MISSING_DIAGONAL, "Missing diagonal on row " + std::to_string(k + 1));
  }
}

void SSOR::apply(const Vec& b, Vec& x) {
  // SSOR.java:143-194: x on entry is the starting iterate.
  const int n = F.n;
  for (int i = 0; i < n; ++i) xx[i] = x[i];
  for (int i = 0; i < n; ++i) {
    double sigma = 0;
    for (int j = F.rowptr[i]; j < diagind[i]; ++j) sigma += F.data[j] * xx[F.col[j]];
    for (int j = diagind[i] + 1; j < F.rowptr[i + 1]; ++j) sigma += F.data[j] * x[F.col[j]];
    sigma = (b[i] - sigma) / F.data[diagind[i]];
    xx[i] = x[i] + omegaF * (sigma - x[i]);
  }
  if (!reverse) {
    for (int i = 0; i < n; ++i) x[i] = xx[i];
    return;
  }
  for (int i = n - 1; i >= 0; --i) {
    double sigma = 0;
    for (int j = F.rowptr[i]; j < diagind[i]; ++j) sigma += F.data[j] * xx[F.col[j]];
    for (int j = diagind[i] + 1; j < F.rowptr[i + 1]; ++j) sigma += F.data[j] * x[F.col[j]];
    sigma = (b[i] - sigma) / F.data[diagind[i]];
    x[i] = xx[i] + omegaR * (sigma - xx[i]);
  }
}

// -------------------------------------------------------------- Krylov ----
void cg_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& iter) {
  // CG.java:58-87
  const int n = A.n;
  Vec p(n, 0.0), z(n, 0.0), q(n, 0.0), r(n, 0.0);
  double alpha = 0, beta = 0, rho = 0, rho_1 = 0;
  vset(r, b);
  A.multAdd(-1, x, r);
  for (iter.setFirst(); !iter.converged(r); iter.next()) {
    M.apply(r, z);
    rho = dot(r, z);
    if (iter.isFirst()) vset(p, z);
    else {
      beta = rho / rho_1;
      vscale(p, beta);
      vadd(p, z);
    }
    A.mult(p, q);
    alpha = rho / dot(p, q);
    vadd(x, alpha, p);
    vadd(r, -alpha, q);
    rho_1 = rho;
  }
}

void bicgstab_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& iter) {
  // BiCGstab.java:65-116
  const int n = A.n;
  Vec p(n, 0.0), s(n, 0.0), phat(n, 0.0), shat(n, 0.0), t(n, 0.0), v(n, 0.0), temp(n, 0.0), r(n, 0.0),
      rtilde(n, 0.0);
  double rho_1 = 1, rho_2 = 1, alpha = 1, beta = 1, omega = 1;
  vset(r, b);
  A.multAdd(-1, x, r);
  vset(rtilde, r);
  for (iter.setFirst(); !iter.converged(r); iter.next()) {
    rho_1 = dot(rtilde, r);
    if (rho_1 == 0) throw Failure(ST_NOT_CONVERGED_BREAKDOWN, "rho", iter.residual, iter.iter);
    if (omega == 0) throw Failure(ST_NOT_CONVERGED_BREAKDOWN, "omega", iter.residual, iter.iter);
    if (iter.isFirst()) vset(p, r);
    else {
      beta = (rho_1 / rho_2) * (alpha / omega);
      vset(temp, -omega, v);
      vadd(temp, p);
      vset(p, r);
      vadd(p, beta, temp);
    }
    M.apply(p, phat);
    A.mult(phat, v);
    alpha = rho_1 / dot(rtilde, v);
    vset(s, r);
    vadd(s, -alpha, v);
    if (iter.converged(s)) {
      vadd(x, alpha, phat);
      return;
    }
    M.apply(s, shat);
    A.mult(shat, t);
    omega = dot(t, s) / dot(t, t);
    vadd(x, alpha, phat);
    vadd(x, omega, shat);
    vset(r, s);
    vadd(r, -omega, t);
    rho_2 = rho_1;
  }
}

// GivensRotation (mtj/src/no/uib/cipr/matrix/GivensRotation.java:42-92)
struct Givens {
  double c = 1, s = 0;
  Givens() {}
  Givens(double x, double y) {
    double roe = std::fabs(x) > std::fabs(y) ? x : y;
    double scale = std::fabs(x) + std::fabs(y);
    if (scale != 0) {
      double xs = x / scale, ys = y / scale;
      double r = scale * std::sqrt(xs * xs + ys * ys);
      if (roe < 0) r *= -1;
      c = x / r;
      s = y / r;
    } else {
      c = 1;
      s = 0;
    }
  }
  // apply(Matrix H, column, i1, i2), :72-76
  void apply(double* H, int ldh, int column, int i1, int i2) const {
    double& a = H[i1 + column * ldh];
    double& b = H[i2 + column * ldh];
    double temp = c * a + s * b;
    b = -s * a + c * b;
    a = temp;
  }
  // apply(Vector x, i1, i2), :88-92
  void apply(Vec& x, int i1, int i2) const {
    double temp = c * x[i1] + s * x[i2];
    x[i2] = -s * x[i1] + c * x[i2];
    x[i1] = temp;
  }
};

void gmres_solve(const CompRowMatrix& A, const Vec& b, Vec& x, Preconditioner& M, IterationMonitor& iter,
                 int restart) {
  // GMRES.java:99-176 (left preconditioned, modified Gram-Schmidt)
  if (restart <= 0) throw Failure(ST_BAD_ARG, "restart must be a positive integer");
  const int n = A.n;
  Vec w(n, 0.0), u(n, 0.0), r(n, 0.0);
  Vec s(restart + 1, 0.0);
  const int ldh = restart + 1;
  std::vector<double> H((size_t)(restart + 1) * restart, 0.0);
  std::vector<Givens> rotation(restart + 1);
  std::vector<Vec> v(restart + 1, Vec(n, 0.0));

  vset(u, b);
  A.multAdd(-1, x, u);
  M.apply(u, r);
  double normr = norm2(r);
  M.apply(b, u);

  for (iter.setFirst(); !iter.converged(r); iter.next()) {
    vset(v[0], 1 / normr, r);
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = normr;
    int i = 0;
    for (; i < restart && !iter.converged(std::fabs(s[i])); i++, iter.next()) {
      A.mult(v[i], u);
      M.apply(u, w);
      for (int k = 0; k <= i; k++) {
        H[k + i * ldh] = dot(w, v[k]);
        vadd(w, -H[k + i * ldh], v[k]);
      }
      H[i + 1 + i * ldh] = norm2(w);
      vset(v[i + 1], 1. / H[i + 1 + i * ldh], w);
      for (int k = 0; k < i; ++k) rotation[k].apply(H.data(), ldh, i, k, k + 1);
      rotation[i] = Givens(H[i + i * ldh], H[i + 1 + i * ldh]);
      rotation[i].apply(H.data(), ldh, i, i, i + 1);
      rotation[i].apply(s, i, i + 1);
    }
    // new UpperTriangDenseMatrix(H, i, false).solve(s, s) -> LAPACK dtrtrs
    if (dtrtrs_upper(i, H.data(), ldh, s.data()) != 0) throw Failure(ST_SINGULAR, "GMRES Hessenberg singular");
    for (int j = 0; j < i; j++) vadd(x, s[j], v[j]);
    vset(u, b);
    A.multAdd(-1, x, u);
    M.apply(u, r);
    normr = norm2(r);
  }
}

// ---------------------------------------------------------- dense LU ----
// Restated from the published netlib LAPACK/BLAS reference algorithms
// (dgetf2, dgetrs, dlaswp, dtrsm, dger, dscal, idamax, dgemm).
int dgesv(int n, int nrhs, double* A, int lda, int* ipiv, double* B, int ldb) {
  int info = 0;
  // dgetf2: unblocked right-looking LU with partial pivoting
  for (int j = 0; j < n; ++j) {
    // idamax over A(j:n-1, j): first index of the largest |a|
    int jp = j;
    double amax = std::fabs(A[j + j * lda]);
    for (int i = j + 1; i < n; ++i) {
      double a = std::fabs(A[i + j * lda]);
      if (a > amax) { amax = a; jp = i; }
    }
    ipiv[j] = jp;
    if (A[jp + j * lda] != 0.0) {
      if (jp != j)
        for (int c = 0; c < n; ++c) std::swap(A[j + c * lda], A[jp + c * lda]);
      if (j < n - 1) {
        double rp = 1.0 / A[j + j * lda];
        for (int i = j + 1; i < n; ++i) A[i + j * lda] *= rp;
      }
    } else if (info == 0) {
      info = j + 1;
    }
    if (j < n - 1) {
      // dger: A(j+1:, j+1:) += x * y' with alpha = -1
      for (int c = j + 1; c < n; ++c) {
        double yv = A[j + c * lda];
        if (yv != 0.0) {
          double temp = -1.0 * yv;
          for (int i = j + 1; i < n; ++i) A[i + c * lda] += A[i + j * lda] * temp;
        }
      }
    }
  }
  if (info != 0) return info;
  // dgetrs: dlaswp then dtrsm(L, Lower, N, Unit) then dtrsm(L, Upper, N, NonUnit)
  for (int j = 0; j < n; ++j)
    if (ipiv[j] != j)
      for (int c = 0; c < nrhs; ++c) std::swap(B[j + c * ldb], B[ipiv[j] + c * ldb]);
  for (int c = 0; c < nrhs; ++c) {
    double* bc = B + c * ldb;
    for (int k = 0; k < n; ++k)
      if (bc[k] != 0.0)
        for (int i = k + 1; i < n; ++i) bc[i] -= bc[k] * A[i + k * lda];
    for (int k = n - 1; k >= 0; --k)
      if (bc[k] != 0.0) {
        bc[k] = bc[k] / A[k + k * lda];
        for (int i = 0; i < k; ++i) bc[i] -= bc[k] * A[i + k * lda];
      }
  }
  return 0;
}

void dgemm_nn_add(int m, int n, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int l = 0; l < k; ++l) {
      double bl = B[l + j * ldb];
      if (bl != 0.0) {
        double temp = 1.0 * bl;
        for (int i = 0; i < m; ++i) C[i + j * ldc] += temp * A[i + l * lda];
      }
    }
}

int dtrtrs_upper(int n, const double* A, int lda, double* b) {
  for (int i = 0; i < n; ++i)
    if (A[i + i * lda] == 0.0) return i + 1;
  for (int k = n - 1; k >= 0; --k)
    if (b[k] != 0.0) {
      b[k] = b[k] / A[k + k * lda];
      for (int i = 0; i < k; ++i) b[i] -= b[k] * A[i + k * lda];
    }
  return 0;
}

}  // namespace orc
