// Oracle (test infrastructure only): C entry points of the CPU restatement,
// loaded with ctypes by tests/, the smoke check and bench.py's CPU-baseline
// leg.  Never linked into the product library.
#include <cstring>
#include <memory>

#include "mesh.hpp"
#include "mtj.hpp"
#include "physics.hpp"

using namespace orc;

namespace {
void put_err(char* err, int errlen, const char* msg) {
  if (err && errlen > 0) {
    std::strncpy(err, msg, errlen - 1);
    err[errlen - 1] = 0;
  }
}
CompRowMatrix make_csr(int n, int nnz, const int* rowptr, const int* col, const double* val) {
  CompRowMatrix A;
  A.n = n;
  A.rowptr.assign(rowptr, rowptr + n + 1);
  A.col.assign(col, col + nnz);
  if (val) A.data.assign(val, val + nnz);
  else A.data.assign(nnz, 0.0);
  return A;
}
std::unique_ptr<Preconditioner> make_pc(int precond, double omegaF, double omegaR, int reverse) {
  switch (precond) {
    case P_NONE: return std::unique_ptr<Preconditioner>(new IdentityPreconditioner());
    case P_DIAGONAL: return std::unique_ptr<Preconditioner>(new DiagonalPreconditioner());
    case P_ILU: return std::unique_ptr<Preconditioner>(new ILU());
    case P_SSOR: {
      auto* s = new SSOR();
      s->omegaF = omegaF;
      s->omegaR = omegaR;
      s->reverse = reverse != 0;
      return std::unique_ptr<Preconditioner>(s);
    }
    case P_AMG: return std::unique_ptr<Preconditioner>(new AMG());
  }
  throw Failure(ST_UNSUPPORTED, "preconditioner not available in the oracle");
}
}  // namespace

extern "C" {

int orc_solve(int method, int precond, int n, int nnz, const int* rowptr, const int* col, const double* val,
              const double* b, double* x, double rtol, double atol, double dtol, int maxit, int restart,
              double omegaF, double omegaR, int* iters, double* resid, double* history, int hist_cap, int* hist_len,
              char* err, int errlen) {
  std::vector<double> hist;
  IterationMonitor it;
  it.rtol = rtol;
  it.atol = atol;
  it.dtol = dtol;
  it.maxIter = maxit;
  it.history = &hist;
  int status = 0;
  try {
    CompRowMatrix A = make_csr(n, nnz, rowptr, col, val);
    Vec vb(b, b + n), vx(x, x + n);
    auto M = make_pc(precond, omegaF, omegaR, 1);
    M->setMatrix(A);
    switch (method) {
      case M_CG: cg_solve(A, vb, vx, *M, it); break;
      case M_BICGSTAB: bicgstab_solve(A, vb, vx, *M, it); break;
      case M_GMRES: gmres_solve(A, vb, vx, *M, it, restart); break;
      default: throw Failure(ST_UNSUPPORTED, "unknown method");
    }
    std::memcpy(x, vx.data(), sizeof(double) * n);
  } catch (Failure& f) {
    status = f.status;
    put_err(err, errlen, f.what());
  }
  if (iters) *iters = it.iter;
  if (resid) *resid = it.residual;
  if (hist_len) *hist_len = (int)hist.size();
  if (history)
    for (int i = 0; i < (int)hist.size() && i < hist_cap; ++i) history[i] = hist[i];
  return status;
}

// ILU(0) factor + apply / transApply.  LUout (nnz) receives the factors.
int orc_ilu(int n, int nnz, const int* rowptr, const int* col, const double* val, const double* b, double* x,
            int trans, double* LUout, char* err, int errlen) {
  try {
    CompRowMatrix A = make_csr(n, nnz, rowptr, col, val);
    ILU ilu;
    ilu.setMatrix(A);
    if (LUout) std::memcpy(LUout, ilu.LU.data.data(), sizeof(double) * nnz);
    if (b && x) {
      Vec vb(b, b + n), vx(n, 0.0);
      if (trans) ilu.transApply(vb, vx);
      else ilu.apply(vb, vx);
      std::memcpy(x, vx.data(), sizeof(double) * n);
    }
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
  return 0;
}

// SSOR.apply with x as the starting iterate (in/out).
int orc_ssor(int n, int nnz, const int* rowptr, const int* col, const double* val, const double* b, double* x,
             double omegaF, double omegaR, int reverse, char* err, int errlen) {
  try {
    CompRowMatrix A = make_csr(n, nnz, rowptr, col, val);
    SSOR s;
    s.omegaF = omegaF;
    s.omegaR = omegaR;
    s.reverse = reverse != 0;
    s.setMatrix(A);
    Vec vb(b, b + n), vx(x, x + n);
    s.apply(vb, vx);
    std::memcpy(x, vx.data(), sizeof(double) * n);
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
  return 0;
}

// kind 0: y = A x; 1: y = alpha A x + y; 2: y = A^T x
int orc_csr_op(int kind, int n, int nnz, const int* rowptr, const int* col, const double* val, double alpha,
               const double* x, double* y) {
  CompRowMatrix A = make_csr(n, nnz, rowptr, col, val);
  Vec vx(x, x + n), vy(y, y + n);
  if (kind == 0) A.mult(vx, vy);
  else if (kind == 1) A.multAdd(alpha, vx, vy);
  else A.transMult(vx, vy);
  std::memcpy(y, vy.data(), sizeof(double) * n);
  return 0;
}

int orc_zero_rows(int n, int nnz, const int* rowptr, const int* col, double* val, double diagonal, int nrows,
                  const int* rows) {
  try {
    CompRowMatrix A = make_csr(n, nnz, rowptr, col, val);
    zeroRows(A, diagonal, std::vector<int>(rows, rows + nrows));
    std::memcpy(val, A.data.data(), sizeof(double) * nnz);
  } catch (Failure& f) {
    return f.status;
  }
  return 0;
}

int orc_dgesv(int n, int nrhs, double* A, double* B) {
  std::vector<int> ipiv(n);
  return dgesv(n, nrhs, A, n, ipiv.data(), B, n);
}

void* orc_mesh_create(int dim, int ni, int nj, int nk, const double* coords, double x0, double y0, double z0,
                      double dx, double dy, double dz, const double* perm, int* status, char* err, int errlen) {
  try {
    Mesh* m = new Mesh(build_structured_mesh(dim, ni, nj, nk, coords, x0, y0, z0, dx, dy, dz));
    if (perm) std::memcpy(m->K6.data(), perm, sizeof(double) * 6 * m->numElements());
    *status = 0;
    return m;
  } catch (Failure& f) {
    *status = f.status;
    put_err(err, errlen, f.what());
    return nullptr;
  }
}

void orc_mesh_destroy(void* h) { delete (Mesh*)h; }

int orc_mesh_mpfa(void* h, double continuity, int tpfa, char* err, int errlen) {
  try {
    if (tpfa == 1) compute_tpfa(*(Mesh*)h);
    else if (tpfa == 2) compute_mpfa_l(*(Mesh*)h);
    else compute_mpfa_o(*(Mesh*)h, continuity);
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
  return 0;
}

int orc_mesh_test(void* h, char* err, int errlen) {
  try {
    test_mesh(*(Mesh*)h);
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
  return 0;
}

int orc_mesh_counts(void* h, long long* counts) {
  Mesh* m = (Mesh*)h;
  long long md = 0;
  for (auto& l : m->MD) md += (long long)l.size();
  counts[0] = m->numElements();
  counts[1] = m->numConnections();
  counts[2] = md;
  counts[3] = m->numPoints();
  counts[4] = (long long)m->iarea.size();
  return 0;
}

// centers (3n), volumes (n), points (3 per point), inormal/icenter (3 per
// interface), iarea (per interface); any may be NULL.
int orc_mesh_geometry(void* h, double* centers, double* volumes, double* points, double* inormal, double* icenter,
                      double* iarea) {
  Mesh* m = (Mesh*)h;
  for (int e = 0; e < m->numElements(); ++e) {
    if (centers) {
      centers[3 * e] = m->ecenter[e].x;
      centers[3 * e + 1] = m->ecenter[e].y;
      centers[3 * e + 2] = m->ecenter[e].z;
    }
    if (volumes) volumes[e] = m->evolume[e];
  }
  if (points)
    for (int p = 0; p < m->numPoints(); ++p) {
      points[3 * p] = m->point[p].x;
      points[3 * p + 1] = m->point[p].y;
      points[3 * p + 2] = m->point[p].z;
    }
  for (size_t f = 0; f < m->iarea.size(); ++f) {
    if (inormal) {
      inormal[3 * f] = m->inormal[f].x;
      inormal[3 * f + 1] = m->inormal[f].y;
      inormal[3 * f + 2] = m->inormal[f].z;
    }
    if (icenter) {
      icenter[3 * f] = m->icenter[f].x;
      icenter[3 * f + 1] = m->icenter[f].y;
      icenter[3 * f + 2] = m->icenter[f].z;
    }
    if (iarea) iarea[f] = m->iarea[f];
  }
  return 0;
}

int orc_mesh_connections(void* h, int* conn) {
  Mesh* m = (Mesh*)h;
  for (int c = 0; c < m->numConnections(); ++c) {
    conn[2 * c] = m->connHere[c];
    conn[2 * c + 1] = m->connThere[c];
  }
  return 0;
}

int orc_mesh_md(void* h, int* md_ptr, int* md_elem, double* md_k) {
  Mesh* m = (Mesh*)h;
  int pos = 0;
  md_ptr[0] = 0;
  for (int c = 0; c < m->numConnections(); ++c) {
    for (auto& t : m->MD[c]) {
      md_elem[pos] = t.element;
      md_k[pos] = t.k;
      pos++;
    }
    md_ptr[c + 1] = pos;
  }
  return 0;
}

// Replaces the MD lists (used to feed GPU-computed transmissibilities back).
int orc_mesh_set_md(void* h, const int* md_ptr, const int* md_elem, const double* md_k) {
  Mesh* m = (Mesh*)h;
  for (int c = 0; c < m->numConnections(); ++c) {
    m->MD[c].clear();
    for (int q = md_ptr[c]; q < md_ptr[c + 1]; ++q) m->MD[c].push_back({md_elem[q], md_k[q]});
  }
  return 0;
}

int orc_mesh_pattern(void* h, int which, int* rowptr, int* col, long long* nnz) {
  Mesh* m = (Mesh*)h;
  CompRowMatrix A = which == 0 ? pressure_pattern(*m) : potential_pattern(*m);
  *nnz = A.nnz();
  if (rowptr) std::memcpy(rowptr, A.rowptr.data(), sizeof(int) * (A.n + 1));
  if (col) std::memcpy(col, A.col.data(), sizeof(int) * A.nnz());
  return 0;
}

void* orc_sim_create(void* mesh, const rsg_blackoil* fluid, const rsg_corey* rf, const double* poro,
                     const double* cr, int ns, const rsg_source* src, const rsg_initial* init,
                     const rsg_runspec* spec, int* status, char* err, int errlen) {
  try {
    auto* s = new Simulator(*(Mesh*)mesh, *fluid, *rf, poro, cr, ns, src, *init, *spec);
    *status = 0;
    return s;
  } catch (Failure& f) {
    *status = f.status;
    put_err(err, errlen, f.what());
    return nullptr;
  }
}

void* orc_sim_create_cubic(void* mesh, const rsg_cubic_fluid* fluid, const rsg_corey* rf, const double* poro,
                           const double* cr, int ns, const rsg_source* src, const rsg_initial* init,
                           const rsg_runspec* spec, int* status, char* err, int errlen) {
  // the black-oil record carries the component count, molecular weights and
  // grouping; its functions are not evaluated
  rsg_blackoil carrier{};
  carrier.nc = fluid->nc;
  for (int i = 0; i < fluid->nc && i < RSG_MAX_COMPONENTS; ++i) {
    carrier.molecular_weight[i] = fluid->Mw[i];
    carrier.group[i] = i == 0 ? 0 : 1;
  }
  rsg_function one{};
  one.kind = RSG_FN_CONSTANT;
  one.dim = 3;
  one.value = 1.0;
  rsg_function zero = one;
  zero.value = 0.0;
  carrier.water_density = fluid->water_density;
  carrier.water_viscosity = fluid->water_viscosity;
  carrier.water_enthalpy = zero;
  carrier.bubble_point = zero;
  carrier.dew_point = zero;
  carrier.oil_density = carrier.gas_density = one;
  carrier.oil_viscosity = carrier.gas_viscosity = one;
  carrier.oil_enthalpy = carrier.gas_enthalpy = zero;
  try {
    auto* s = new Simulator(*(Mesh*)mesh, carrier, *rf, poro, cr, ns, src, *init, *spec, fluid);
    *status = 0;
    return s;
  } catch (Failure& f) {
    *status = f.status;
    put_err(err, errlen, f.what());
    return nullptr;
  }
}

void orc_sim_destroy(void* s) { delete (Simulator*)s; }

int orc_sim_step(void* h, double dt, rsg_step_info* info, char* err, int errlen) {
  Simulator* s = (Simulator*)h;
  try {
    s->step(dt, info);
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    if (info) info->status = f.status;
    return f.status;
  }
  return 0;
}

void orc_cubic_roots(double a0, double a1, double a2, double* z) { cubic_roots_kat(a0, a1, a2, z); }

// phases: [3][6 + 2 nc][n] as rsg_cubic_phase_state
int orc_cubic_phase_state(const rsg_cubic_fluid* fl, int n, const double* p, const double* T, const double* N,
                          double* phases, int* iterations, char* err, int errlen) {
  const int nc = fl->nc, nf = 6 + 2 * nc;
  try {
    Function wden(fl->water_density), wvis(fl->water_viscosity);
    for (int i = 0; i < n; ++i) {
      EOSData ph[3];
      double Ni[RSG_MAX_COMPONENTS] = {0};
      for (int nu = 0; nu < nc; ++nu) Ni[nu] = N[(size_t)nu * n + i];
      for (int a = 0; a < 3; ++a) {
        auto at = [&](int f) -> double& { return phases[((size_t)a * nf + f) * n + i]; };
        ph[a].present = at(0) != 0;
        ph[a].V = at(1);
        ph[a].xi = at(2);
        ph[a].dVdp = at(3);
        ph[a].dVdT = at(4);
        ph[a].mu = at(5);
        for (int nu = 0; nu < nc; ++nu) {
          ph[a].N[nu] = at(6 + nu);
          ph[a].dVdN[nu] = at(6 + nc + nu);
        }
      }
      int it = cubic_phase_state(*fl, wden, wvis, p[i], T[i], Ni, ph);
      if (iterations) iterations[i] = it;
      for (int a = 0; a < 3; ++a) {
        auto at = [&](int f) -> double& { return phases[((size_t)a * nf + f) * n + i]; };
        at(0) = ph[a].present ? 1 : 0;
        at(1) = ph[a].V;
        at(2) = ph[a].xi;
        at(3) = ph[a].dVdp;
        at(4) = ph[a].dVdT;
        at(5) = ph[a].mu;
        for (int nu = 0; nu < nc; ++nu) {
          at(6 + nu) = ph[a].N[nu];
          at(6 + nc + nu) = ph[a].dVdN[nu];
        }
      }
    }
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
  return 0;
}

double orc_sim_time(void* h) { return ((Simulator*)h)->time; }

// util/Function.get (nd < 0) or deriv(nd, x) at m points x (m x dim, row major)
int orc_function_eval(const rsg_function* f, int nd, int m, const double* x, double* out) {
  Function fn(*f);
  for (int i = 0; i < m; ++i) out[i] = nd < 0 ? fn.get(x + (size_t)i * f->dim) : fn.deriv(nd, x + (size_t)i * f->dim);
  return 0;
}

// the last step's molar changes before the locks (nc * n)
int orc_sim_last_dn(void* h, double* dN) {
  Simulator* s = (Simulator*)h;
  std::copy(s->dNfull.begin(), s->dNfull.end(), dN);
  return (int)s->dNfull.size();
}

int orc_sim_calculate_dt(void* h, double dt, const rsg_dt_control* c, double* dt_new, rsg_dt_factors* f) {
  *dt_new = ((Simulator*)h)->calculateDt(dt, *c, f);
  return 0;
}

double orc_sim_throughput_factor(void* h, const rsg_dt_control* c) { return ((Simulator*)h)->throughputFactor(*c); }

int orc_sim_step_to(void* h, double end_time, const rsg_dt_control* c, double* dt, rsg_step_to_info* info, char* err,
                    int errlen) {
  try {
    return ((Simulator*)h)->stepTo(end_time, *c, *dt, info);
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    if (info) info->status = f.status;
    return f.status;
  }
}

int orc_sim_set_rock_tables(void* h, const rsg_rock_tables* t, char* err, int errlen) {
  try {
    Simulator* s = (Simulator*)h;
    s->rockFluid.setTables(*t);
    s->calculateSecondaries();
    return 0;
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
}

int orc_sim_retract(void* h) {
  ((Simulator*)h)->retract();
  return 0;
}

int orc_sim_state(void* h, double* p, double* N, double* S) {
  Simulator* s = (Simulator*)h;
  const int n = s->mesh->numElements();
  for (int i = 0; i < n; ++i) {
    if (p) p[i] = s->cv[i].p;
    if (N)
      for (int nu = 0; nu < s->nc; ++nu) N[(size_t)nu * n + i] = s->cv[i].N[nu];
    if (S)
      for (int ph = 0; ph < 3; ++ph) S[(size_t)ph * n + i] = s->cv[i].S[ph];
  }
  return 0;
}

int orc_sim_jacobian(void* h, double* vals, double* rhs) {
  Simulator* s = (Simulator*)h;
  if (vals && !s->lastJ.empty()) std::memcpy(vals, s->lastJ.data(), sizeof(double) * s->lastJ.size());
  if (rhs && !s->lastRhs.empty()) std::memcpy(rhs, s->lastRhs.data(), sizeof(double) * s->lastRhs.size());
  return 0;
}

// AMG hierarchy access for the parity tests.
void* orc_amg_create(int n, int nnz, const int* rowptr, const int* col, const double* val, int* status, char* err,
                     int errlen) {
  try {
    auto* a = new AMG();
    a->setMatrix(make_csr(n, nnz, rowptr, col, val));
    *status = 0;
    return a;
  } catch (Failure& f) {
    *status = f.status;
    put_err(err, errlen, f.what());
    return nullptr;
  }
}

void orc_amg_destroy(void* h) { delete (AMG*)h; }

int orc_amg_levels(void* h) { return (int)((AMG*)h)->L.size(); }

// sizes[0..3] = n, nnz, c (coarse size, 0 on the last level), nnz of I
void orc_amg_level_sizes(void* h, int k, int* sizes) {
  const AMGLevel& l = ((AMG*)h)->L[k];
  sizes[0] = l.A.n;
  sizes[1] = l.A.nnz();
  sizes[2] = l.c;
  sizes[3] = (int)l.rowind.size();
}

void orc_amg_level_get(void* h, int k, int* rowptr, int* col, double* val, int* pt, int* colptr, int* rowind,
                       double* Idata) {
  const AMGLevel& l = ((AMG*)h)->L[k];
  std::memcpy(rowptr, l.A.rowptr.data(), sizeof(int) * (l.A.n + 1));
  std::memcpy(col, l.A.col.data(), sizeof(int) * l.A.nnz());
  std::memcpy(val, l.A.data.data(), sizeof(double) * l.A.nnz());
  if (pt && !l.pt.empty()) std::memcpy(pt, l.pt.data(), sizeof(int) * l.pt.size());
  if (colptr && !l.colptr.empty()) std::memcpy(colptr, l.colptr.data(), sizeof(int) * l.colptr.size());
  if (rowind && !l.rowind.empty()) std::memcpy(rowind, l.rowind.data(), sizeof(int) * l.rowind.size());
  if (Idata && !l.Idata.empty()) std::memcpy(Idata, l.Idata.data(), sizeof(double) * l.Idata.size());
}

int orc_amg_apply(void* h, const double* b, double* x, int trans, char* err, int errlen) {
  AMG* a = (AMG*)h;
  const int n = a->L[0].A.n;
  try {
    Vec vb(b, b + n), vx(x, x + n);
    if (trans) a->transApply(vb, vx);
    else a->apply(vb, vx);
    std::memcpy(x, vx.data(), sizeof(double) * n);
    return 0;
  } catch (Failure& f) {
    put_err(err, errlen, f.what());
    return f.status;
  }
}

// Test hook: every cell's pressure and moles (N component major) replaced,
// its CV secondaries re-evaluated (CV.calculateSecondaries), and R, dR/dp
// and dR/dN returned, so that the analytic volume derivatives can be checked
// against differences.  The simulator is left at the given state.
int orc_sim_eval_cells(void* h, const double* p, const double* N, double* R, double* dRdp, double* dRdN) {
  Simulator* s = (Simulator*)h;
  const int n = s->mesh->numElements();
  try {
    for (int i = 0; i < n; ++i) {
      s->cv[i].p = p[i];
      for (int nu = 0; nu < s->nc; ++nu) s->cv[i].N[nu] = N[(size_t)nu * n + i];
      s->cvSecondaries(i);
      R[i] = s->cv[i].R;
      dRdp[i] = s->cv[i].dRdp;
      for (int nu = 0; nu < s->nc; ++nu) dRdN[(size_t)nu * n + i] = s->cv[i].dRdN[nu];
    }
  } catch (Failure& f) {
    return f.status;
  }
  return 0;
}

int orc_sim_residual_volume(void* h, double* R, double* dRdp) {
  Simulator* s = (Simulator*)h;
  for (int i = 0; i < s->mesh->numElements(); ++i) {
    if (R) R[i] = s->cv[i].R;
    if (dRdp) dRdp[i] = s->cv[i].dRdp;
  }
  return 0;
}

}  // extern "C"
