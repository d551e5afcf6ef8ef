// Oracle (test infrastructure only): restatement of MTJ's smoothed-
// aggregation AMG preconditioner (mtj/src/no/uib/cipr/matrix/sparse/AMG.java)
// and of the netlib dgetf2/dgetrs pair behind DenseLU (DenseLU.java:83-196).
//
// Two places are restated in an equivalent rather than literal form:
//  * Interpolator.createGalerkinSlow (AMG.java:883-919) forms I'AI one
//    dense column at a time.  Here the same sums are taken over the non-zero
//    terms only, in the same order (row i of A in CSR order, column k' of I in
//    ascending row order); terms that are exactly zero cannot change a sum,
//    so every stored value is identical.
//  * Aggregator.enlargeAggregates (AMG.java:540-582) walks N_i, a
//    java.util.HashSet, whose iteration order follows the HashMap bucket
//    layout (and its tree bins).  That order only decides ties between
//    aggregates of equal overlap; it is restated as ascending node index.
#include <algorithm>
#include <cmath>

#include "mtj.hpp"

namespace orc {

int dgetf2(int n, double* A, int lda, int* ipiv) {
  // dgetf2 for m == n: idamax pivot, row swap, reciprocal scaling, dger
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int jp = j;
    double amax = std::fabs(A[j + j * lda]);
    for (int i = j + 1; i < n; ++i) {
      double a = std::fabs(A[i + j * lda]);
      if (a > amax) {
        amax = a;
        jp = i;
      }
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
    if (j < n - 1)
      for (int c = j + 1; c < n; ++c) {
        double yv = A[j + c * lda];
        if (yv != 0.0) {
          double temp = -1.0 * yv;
          for (int i = j + 1; i < n; ++i) A[i + c * lda] += A[i + j * lda] * temp;
        }
      }
  }
  return info;
}

void dgetrs(bool trans, int n, const double* A, int lda, const int* ipiv, double* b) {
  if (!trans) {
    // dlaswp (forward), dtrsm(L, Lower, N, Unit), dtrsm(L, Upper, N, NonUnit)
    for (int j = 0; j < n; ++j)
      if (ipiv[j] != j) std::swap(b[j], b[ipiv[j]]);
    for (int k = 0; k < n; ++k)
      if (b[k] != 0.0)
        for (int i = k + 1; i < n; ++i) b[i] -= b[k] * A[i + k * lda];
    for (int k = n - 1; k >= 0; --k)
      if (b[k] != 0.0) {
        b[k] = b[k] / A[k + k * lda];
        for (int i = 0; i < k; ++i) b[i] -= b[k] * A[i + k * lda];
      }
    return;
  }
  // dtrsm(L, Upper, T, NonUnit), dtrsm(L, Lower, T, Unit), dlaswp (backward)
  for (int i = 0; i < n; ++i) {
    double temp = b[i];
    for (int k = 0; k < i; ++k) temp -= A[k + i * lda] * b[k];
    temp = temp / A[i + i * lda];
    b[i] = temp;
  }
  for (int i = n - 1; i >= 0; --i) {
    double temp = b[i];
    for (int k = i + 1; k < n; ++k) temp -= A[k + i * lda] * b[k];
    b[i] = temp;
  }
  for (int j = n - 1; j >= 0; --j)
    if (ipiv[j] != j) std::swap(b[j], b[ipiv[j]]);
}

namespace {

int find_diag(const CompRowMatrix& A, int i) {
  int lo = A.rowptr[i], hi = A.rowptr[i + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    if (A.col[mid] < i) lo = mid + 1;
    else if (A.col[mid] > i) hi = mid - 1;
    else return mid;
  }
  return -1;
}

// Small ordered accumulator: keys in order of first appearance, one running
// sum per key, so every key's additions happen in the caller's order.
struct Acc {
  std::vector<int> key;
  std::vector<double> val;
  int slot(int k) {
    for (size_t q = 0; q < key.size(); ++q)
      if (key[q] == k) return (int)q;
    key.push_back(k);
    val.push_back(0.0);
    return (int)key.size() - 1;
  }
  void clear() {
    key.clear();
    val.clear();
  }
};

struct Coarsening {
  std::vector<int> pt;
  int c = 0;
  std::vector<int> colptr, rowind;
  Vec Idata;
  CompRowMatrix Ac;
};

// Aggregator (AMG.java:402-641) followed by Interpolator (:650-919) for one
// level; returns false when no aggregate was formed.
bool coarsen(const CompRowMatrix& A, double eps, double omega, Coarsening& out) {
  const int n = A.n;
  // findDiagonalIndices (:446-461)
  std::vector<int> diagind(n);
  for (int i = 0; i < n; ++i) {
    diagind[i] = find_diag(A, i);
    if (diagind[i] < 0)
      throw Failure(ST_MISSING_DIAGONAL, "Matrix is missing a diagonal entry on row " + std::to_string(i + 1));
  }
  // findNodeNeighborhood (:470-494): N_i in CSR (ascending) order
  std::vector<std::vector<int>> N(n);
  for (int i = 0; i < n; ++i) {
    double aii = A.data[diagind[i]];
    for (int j = A.rowptr[i]; j < A.rowptr[i + 1]; ++j) {
      double aij = A.data[j];
      double ajj = A.data[diagind[A.col[j]]];
      if (std::fabs(aij) >= eps * std::sqrt(aii * ajj)) N[i].push_back(A.col[j]);
    }
  }
  auto in_N = [&](int i, int j) { return std::binary_search(N[i].begin(), N[i].end(), j); };
  // createInitialR (:500-518)
  std::vector<char> R(n);
  for (int i = 0; i < n; ++i) {
    bool off = false;
    for (int j = A.rowptr[i]; j < A.rowptr[i + 1]; ++j)
      if (A.col[j] != i && A.data[j] != 0) {
        off = true;
        break;
      }
    R[i] = off;
  }
  // createInitialAggregates (:524-548)
  std::vector<std::vector<int>> C;
  for (int i = 0; i < n; ++i) {
    if (!R[i]) continue;
    bool free = true;
    for (int j : N[i]) free &= (bool)R[j];
    if (free) {
      C.push_back(N[i]);
      for (int j : N[i]) R[j] = false;
    }
  }
  // enlargeAggregates (:554-600): belong from the initial aggregates
  std::vector<int> belong(n, -1);
  for (int k = 0; k < (int)C.size(); ++k)
    for (int j : C[k]) belong[j] = k;  // aggregates of phase one are disjoint
  std::vector<std::pair<int, int>> joins;
  {
    std::vector<int> intersect(C.size(), 0), touched;
    for (int i = 0; i < n; ++i) {
      if (!R[i]) continue;
      for (int k : touched) intersect[k] = 0;
      touched.clear();
      int largest = 0, maxValue = 0;
      for (int j : N[i]) {
        int k = belong[j];
        if (k < 0) continue;
        if (intersect[k]++ == 0) touched.push_back(k);
        if (intersect[k] > maxValue) {
          largest = k;
          maxValue = intersect[largest];
        }
      }
      if (maxValue > 0) {
        R[i] = false;
        joins.push_back({largest, i});
      }
    }
  }
  for (auto& jn : joins) C[jn.first].push_back(jn.second);
  // createFinalAggregates (:606-628)
  for (int i = 0; i < n; ++i) {
    if (!R[i]) continue;
    std::vector<int> Cn;
    for (int j : N[i])
      if (R[j]) {
        R[j] = false;
        Cn.push_back(j);
      }
    if (!Cn.empty()) C.push_back(Cn);
  }
  if (C.empty()) return false;
  const int c = (int)C.size();
  // createTentativeProlongation (:699-709)
  std::vector<int> pt(n, -1);
  for (int i = 0; i < c; ++i)
    for (int j : C[i]) pt[j] = i;
  // createSmoothedProlongation (:810-876), one row of P at a time
  std::vector<std::vector<std::pair<int, double>>> Pcol(c);
  Acc dot;
  for (int i = 0; i < n; ++i) {
    if (pt[i] == -1) continue;
    dot.clear();
    double weakAij = 0;
    for (int j = A.rowptr[i]; j < A.rowptr[i + 1]; ++j) {
      if (pt[A.col[j]] == -1) continue;
      double aij = A.data[j];
      if (aij != 0 && !in_N(i, A.col[j])) {
        weakAij += aij;
        continue;
      }
      int s = dot.slot(pt[A.col[j]]);
      dot.val[s] += aij;
    }
    int d = dot.slot(pt[i]);
    dot.val[d] -= weakAij;
    double scale = -omega / A.data[diagind[i]];
    for (auto& v : dot.val) v *= scale;
    dot.val[d]++;
    for (size_t q = 0; q < dot.key.size(); ++q)
      if (dot.val[q] != 0) Pcol[dot.key[q]].push_back({i, dot.val[q]});
  }
  // createInterpolationMatrix (:732-749): CompColMatrix, rows sorted per column
  out.colptr.assign(c + 1, 0);
  for (int k = 0; k < c; ++k) out.colptr[k + 1] = out.colptr[k] + (int)Pcol[k].size();
  out.rowind.resize(out.colptr[c]);
  out.Idata.resize(out.colptr[c]);
  for (int k = 0; k < c; ++k) {
    auto& col = Pcol[k];  // rows were appended in ascending order
    for (size_t q = 0; q < col.size(); ++q) {
      out.rowind[out.colptr[k] + q] = col[q].first;
      out.Idata[out.colptr[k] + q] = col[q].second;
    }
  }
  // rows of I (for A*I): entries of row i in ascending column order
  std::vector<std::vector<std::pair<int, double>>> Irow(n);
  for (int k = 0; k < c; ++k)
    for (int q = out.colptr[k]; q < out.colptr[k + 1]; ++q) Irow[out.rowind[q]].push_back({k, out.Idata[q]});
  // createGalerkinSlow (:883-919) over the non-zero terms: B = A*I row by
  // row, then I'*B column of I by column of I
  std::vector<std::vector<std::pair<int, double>>> B(n);
  Acc acc;
  for (int i = 0; i < n; ++i) {
    acc.clear();
    for (int j = A.rowptr[i]; j < A.rowptr[i + 1]; ++j) {
      double aij = A.data[j];
      for (auto& e : Irow[A.col[j]]) {
        double t = aij * e.second;
        int s = acc.slot(e.first);
        acc.val[s] += t;
      }
    }
    for (size_t q = 0; q < acc.key.size(); ++q)
      if (acc.val[q] != 0) B[i].push_back({acc.key[q], acc.val[q]});
  }
  std::vector<std::vector<int>> rows(c);
  std::vector<std::vector<double>> vals(c);
  for (int kp = 0; kp < c; ++kp) {
    acc.clear();
    for (int q = out.colptr[kp]; q < out.colptr[kp + 1]; ++q) {
      const int i = out.rowind[q];
      const double w = out.Idata[q];
      for (auto& e : B[i]) {
        double t = w * e.second;
        int s = acc.slot(e.first);
        acc.val[s] += t;
      }
    }
    std::vector<std::pair<int, double>> row;
    for (size_t q = 0; q < acc.key.size(); ++q)
      if (acc.val[q] != 0) row.push_back({acc.key[q], acc.val[q]});
    std::sort(row.begin(), row.end());
    for (auto& e : row) {
      rows[kp].push_back(e.first);
      vals[kp].push_back(e.second);
    }
  }
  out.Ac = CompRowMatrix::from_rows(c, rows);
  for (int kp = 0; kp < c; ++kp)
    for (size_t q = 0; q < rows[kp].size(); ++q) out.Ac.data[out.Ac.rowptr[kp] + q] = vals[kp][q];
  out.pt = std::move(pt);
  out.c = c;
  return true;
}

}  // namespace

void AMG::setMatrix(const CompRowMatrix& A0) {
  // AMG.java:224-286
  L.clear();
  std::vector<CompRowMatrix> Al{A0};
  std::vector<Coarsening> Cl;
  for (int k = 0; Al[k].n > min; ++k) {
    double eps = 0.08 * std::pow(0.5, k);
    Coarsening co;
    if (!coarsen(Al[k], eps, omega, co)) break;
    Al.push_back(co.Ac);
    Cl.push_back(std::move(co));
  }
  const int m = (int)Al.size();
  L.resize(m);
  for (int k = 0; k < m; ++k) {
    L[k].A = Al[k];
    const int n = Al[k].n;
    L[k].u.assign(n, 0.0);
    L[k].f.assign(n, 0.0);
    L[k].r.assign(n, 0.0);
    if (k < m - 1) {
      L[k].pt = Cl[k].pt;
      L[k].c = Cl[k].c;
      L[k].colptr = Cl[k].colptr;
      L[k].rowind = Cl[k].rowind;
      L[k].Idata = Cl[k].Idata;
      L[k].pre.omegaF = omegaPreF;
      L[k].pre.omegaR = omegaPreR;
      L[k].pre.reverse = true;
      L[k].post.omegaF = omegaPostF;
      L[k].post.omegaR = omegaPostR;
      L[k].post.reverse = true;
      L[k].pre.setMatrix(Al[k]);
      L[k].post.setMatrix(Al[k]);
    }
  }
  // DenseLU of the coarsest operator (DenseMatrix(Matrix) copy, dgetrf)
  const CompRowMatrix& Ac = Al[m - 1];
  nc = Ac.n;
  lu.assign((size_t)nc * nc, 0.0);
  for (int i = 0; i < nc; ++i)
    for (int q = Ac.rowptr[i]; q < Ac.rowptr[i + 1]; ++q) lu[i + (size_t)Ac.col[q] * nc] = Ac.data[q];
  piv.assign(nc, 0);
  singular = dgetf2(nc, lu.data(), nc, piv.data()) > 0;
}

void AMG::directSolve() {
  // AMG.java:315-323
  AMGLevel& c = L.back();
  c.u = c.f;
  if (singular) throw Failure(ST_SINGULAR, "MatrixSingularException: coarsest AMG operator is singular");
  dgetrs(transpose, nc, lu.data(), nc, piv.data(), c.u.data());
}

void AMG::cycle(int k) {
  // AMG.java:288-313
  const int m = (int)L.size();
  if (k == m - 1) {
    directSolve();
    return;
  }
  AMGLevel& l = L[k];
  AMGLevel& nx = L[k + 1];
  for (int i = 0; i < nu1; ++i) l.pre.apply(l.f, l.u);  // preRelax (:325-331)
  std::fill(nx.u.begin(), nx.u.end(), 0.0);
  l.r = l.f;
  l.A.multAdd(-1, l.u, l.r);
  // I.transMult(r, f_{k+1}) (CompColMatrix.java:299-316)
  for (int j = 0; j < l.c; ++j) {
    double dot = 0;
    for (int q = l.colptr[j]; q < l.colptr[j + 1]; ++q) dot += l.Idata[q] * l.r[l.rowind[q]];
    nx.f[j] = dot;
  }
  for (int i = 0; i < gamma; ++i) cycle(k + 1);
  // I.multAdd(u_{k+1}, u_k) (CompColMatrix.java:277-296 with alpha 1)
  for (int j = 0; j < l.c; ++j)
    for (int q = l.colptr[j]; q < l.colptr[j + 1]; ++q) l.u[l.rowind[q]] += l.Idata[q] * nx.u[j];
  for (int i = 0; i < nu2; ++i) l.post.apply(l.f, l.u);  // postRelax (:333-339)
}

void AMG::apply(const Vec& b, Vec& x) {
  L[0].u = x;
  L[0].f = b;
  transpose = false;
  cycle(0);
  x = L[0].u;
}

void AMG::transApply(const Vec& b, Vec& x) {
  L[0].u = x;
  L[0].f = b;
  transpose = true;
  cycle(0);
  x = L[0].u;
}

}  // namespace orc
