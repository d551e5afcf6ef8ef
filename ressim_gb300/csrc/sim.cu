// RS pressure step on the GPU: per-cell property chain (field/CV.java:375-550
// with fluid/WaterEquationOfState.java:71-129, fluid/BlackOilEquationOfState.java:168-547,
// rock/CoreyRockFluid.java:84-141, util/LookupTable.java:202-430), per-connection
// Darcy fluxes (field/CS.java:94-170), the pressure Jacobian
// (numerics/Discretisation.java:365-561), LinearSolver.solve
// (numerics/LinearSolver.java:244-294), the pressure update and Newton test
// (Discretisation.java:280-359), and the explicit molar-mass update
// (Discretisation.java:769-919).  Field initialisation by local volume
// balance (field/Field.java:260-447) runs one thread per cell.
//
// Every sum that RS accumulates over connections is gathered per row in
// ascending connection order, so the assembled Jacobian, residual and mass
// changes equal the sequential Java loops without atomics.
#include <algorithm>
#include <atomic>
#include <set>
#include <thread>
#include <cstring>
#include <limits>
#include <cmath>

#include "dual.cuh"
#include <cudaTypedefs.h>

#include "mesh.cuh"

namespace rsg {

namespace {

constexpr double G_ACC = 9.81;  // util/Constants.java:18
constexpr int NCM = RSG_MAX_COMPONENTS;

struct DFunc {
  int kind, dim;
  double value;
  int n[3];
  const double* coord[3];
  double offset[3], delta[3];
  const double* data;
};

__device__ int f_index(const DFunc& f, int d, double x) {
  if (f.kind == RSG_FN_EVEN_TABLE) {
    // EvenLookupTable.getIndex (:164-174)
    int index = (int)((x - f.offset[d]) / f.delta[d]);
    if (index < 0) index = 0;
    else if (index > f.n[d] - 2) index = f.n[d] - 2;
    return index;
  }
  const double* c = f.coord[d];
  const int len = f.n[d];
  if (x <= c[0]) return 0;
  if (x >= c[len - 2]) return len - 2;
  int begin = 0, end = len - 1;
  while (begin <= end) {
    int mid = (end + begin) / 2;
    if (c[mid] < x) begin = mid + 1;
    else end = mid - 1;
  }
  return begin - 1;
}

template <class S>
__device__ S f_weight(const DFunc& f, int d, int index, S x) {
  double mn = f.coord[d][index], mx = f.coord[d][index + 1];
  if (x <= mn) return S(0);
  if (x >= mx) return S(1);
  return (x - mn) / (mx - mn);
}

// LookupTable.evaluate (:217-357); nd = -1 value, else partial derivative.
// S is double, or a dual number carrying derivatives through the weights.
template <class S>
__device__ S f_eval(const DFunc& f, int nd, const S* x) {
  if (f.kind == RSG_FN_CONSTANT) return S(nd < 0 ? f.value : 0.0);
  if (nd >= 0 && !(x[nd] >= f.coord[nd][0] && x[nd] <= f.coord[nd][f.n[nd] - 1])) return S(0);
  const double* D = f.data;
  const int nx = f.n[0], ny = f.n[1];
  if (f.dim == 1) {
    int xi = f_index(f, 0, val(x[0]));
    S xw = f_weight(f, 0, xi, x[0]);
    S phi1, phi2;
    if (nd == -1) {
      phi1 = 1 - xw;
      phi2 = xw;
    } else {
      double dl = f.coord[0][xi + 1] - f.coord[0][xi];
      phi1 = -1 / dl;
      phi2 = 1 / dl;
    }
    return phi1 * D[xi] + phi2 * D[xi + 1];
  }
  if (f.dim == 2) {
    int xi = f_index(f, 0, val(x[0])), yi = f_index(f, 1, val(x[1]));
    S xw = f_weight(f, 0, xi, x[0]), yw = f_weight(f, 1, yi, x[1]);
    S phi1, phi2, phi3, phi4;
    double dl;
    if (nd == -1) {
      phi1 = (1 - xw) * (1 - yw);
      phi2 = xw * (1 - yw);
      phi3 = (1 - xw) * yw;
      phi4 = xw * yw;
    } else if (nd == 0) {
      dl = f.coord[0][xi + 1] - f.coord[0][xi];
      phi1 = (-1 + yw) / dl;
      phi2 = (1 - yw) / dl;
      phi3 = -yw / dl;
      phi4 = yw / dl;
    } else {
      dl = f.coord[1][yi + 1] - f.coord[1][yi];
      phi1 = (-1 + xw) / dl;
      phi2 = -xw / dl;
      phi3 = (1 - xw) / dl;
      phi4 = xw / dl;
    }
    return phi1 * D[xi + yi * nx] + phi2 * D[xi + 1 + yi * nx] + phi3 * D[xi + (yi + 1) * nx] +
           phi4 * D[xi + 1 + (yi + 1) * nx];
  }
  int xi = f_index(f, 0, val(x[0])), yi = f_index(f, 1, val(x[1])), zi = f_index(f, 2, val(x[2]));
  S xw = f_weight(f, 0, xi, x[0]), yw = f_weight(f, 1, yi, x[1]), zw = f_weight(f, 2, zi, x[2]);
  S p1, p2, p3, p4, p5, p6, p7, p8;
  double dl;
  if (nd == -1) {
    p1 = (1 - xw) * (1 - yw) * (1 - zw);
    p2 = xw * (1 - yw) * (1 - zw);
    p3 = (1 - xw) * yw * (1 - zw);
    p4 = xw * yw * (1 - zw);
    p5 = (1 - xw) * (1 - yw) * zw;
    p6 = xw * (1 - yw) * zw;
    p7 = (1 - xw) * yw * zw;
    p8 = xw * yw * zw;
  } else if (nd == 0) {
    dl = f.coord[0][xi + 1] - f.coord[0][xi];
    p1 = -(1 - yw) * (1 - zw) / dl;
    p2 = (1 - yw) * (1 - zw) / dl;
    p3 = -yw * (1 - zw) / dl;
    p4 = yw * (1 - zw) / dl;
    p5 = -(1 - yw) * zw / dl;
    p6 = (1 - yw) * zw / dl;
    p7 = -yw * zw / dl;
    p8 = yw * zw / dl;
  } else if (nd == 1) {
    dl = f.coord[1][yi + 1] - f.coord[1][yi];
    p1 = -(1 - xw) * (1 - zw) / dl;
    p2 = -xw * (1 - zw) / dl;
    p3 = (1 - xw) * (1 - zw) / dl;
    p4 = xw * (1 - zw) / dl;
    p5 = -(1 - xw) * zw / dl;
    p6 = -xw * zw / dl;
    p7 = (1 - xw) * zw / dl;
    p8 = xw * zw / dl;
  } else {
    dl = f.coord[2][zi + 1] - f.coord[2][zi];
    p1 = -(1 - xw) * (1 - yw) / dl;
    p2 = -xw * (1 - yw) / dl;
    p3 = -(1 - xw) * yw / dl;
    p4 = -xw * yw / dl;
    p5 = (1 - xw) * (1 - yw) / dl;
    p6 = xw * (1 - yw) / dl;
    p7 = (1 - xw) * yw / dl;
    p8 = xw * yw / dl;
  }
  const int sxy = nx * ny;
  auto d3 = [&](int a, int b, int c) { return D[a + b * nx + c * sxy]; };
  return p1 * d3(xi, yi, zi) + p2 * d3(xi + 1, yi, zi) + p3 * d3(xi, yi + 1, zi) + p4 * d3(xi + 1, yi + 1, zi) +
         p5 * d3(xi, yi, zi + 1) + p6 * d3(xi + 1, yi, zi + 1) + p7 * d3(xi, yi + 1, zi + 1) +
         p8 * d3(xi + 1, yi + 1, zi + 1);
}

struct DFluid {
  int nc, ngO, ngG;
  int O[NCM], G[NCM];
  double Mw[NCM];
  DFunc wden, wvis, went, bub, dew, oden, gden, ovis, gvis, oent, gent;
};

struct DCorey {
  double Sr[3], n[3], ke[3], cw, cow, cg, cog, aw, aow, ag, aog;
};

// Per-phase EOS record (EquationOfStateData)
template <class S>
struct PhaseT {
  bool present;
  S V, xi, dVdp, dVdT, h, dhdT, mu;
  S N[NCM], dVdN[NCM];
};
using Phase = PhaseT<double>;

template <class S>
__device__ void phase_clear(PhaseT<S>& e, int nc) {
  e.present = false;
  e.V = e.xi = e.dVdp = e.dVdT = e.h = e.dhdT = e.mu = S(0);
  for (int i = 0; i < nc; ++i) e.N[i] = e.dVdN[i] = S(0);
}

template <class S>
__device__ S mole_fraction(const S* N, int nc, int nu) {
  S NT = 0;
  for (int i = 0; i < nc; ++i) NT += N[i];
  return NT > 0 ? N[nu] / NT : S(0);
}

// Flags raised by the property chain (first one wins)
enum { FL_NONE = 0, FL_DRDP = 1, FL_DENSITY = 2, FL_WATER_DERIV = 3, FL_BLACKOIL_CHECK = 4, FL_ENTHALPY = 5, FL_PATTERN = 6,
       FL_NO_WATER = 7, FL_TMA = 8, FL_CUBIC = 16 };  // FL_CUBIC + CUBIC_* code

// S = double for the simulator; a dual number for the adjoint's local derivatives
template <class S>
__device__ void blackoil_state(const DFluid& fl, S p, const S* N, double T, PhaseT<S>* ph, int* flag) {
  const int nc = fl.nc;
  S pT[2] = {p, S(T)};
  {
    PhaseT<S>& w = ph[0];
    S Nw = N[0];
    if (Nw > 0) {
      w.present = true;
      S xiw = f_eval(fl.wden, -1, pT);
      S Vw = Nw / xiw;
      if (xiw <= 0) atomicCAS(flag, 0, FL_DENSITY);
      w.xi = xiw;
      w.V = Vw;
      w.N[0] = Nw;
      S dxiw_dp = f_eval(fl.wden, 0, pT);
      S dxiw_dT = f_eval(fl.wden, 1, pT);
      if (dxiw_dp < 0) atomicCAS(flag, 0, FL_WATER_DERIV);
      w.dVdp = -(Vw / xiw) * dxiw_dp;
      w.dVdT = -(Vw / xiw) * dxiw_dT;
      w.dVdN[0] = 1 / xiw;
      S hw = f_eval(fl.went, -1, pT);
      w.h = hw * xiw;
      S dhw_dT = f_eval(fl.went, 1, pT);
      w.dhdT = dhw_dT * xiw + hw * dxiw_dT;
      w.mu = f_eval(fl.wvis, -1, pT);
    } else
      phase_clear(w, nc);
  }
  PhaseT<S>& oil = ph[1];
  PhaseT<S>& gas = ph[2];
  S No = 0, Ng = 0;
  for (int a = 0; a < fl.ngO; ++a) No += N[fl.O[a]];
  for (int a = 0; a < fl.ngG; ++a) Ng += N[fl.G[a]];
  S NHC = No + Ng;
  S Nt = 0;
  for (int i = 0; i < nc; ++i) Nt += N[i];
  auto inverse_group = [&](S Nop, S Ngp, PhaseT<S>& e) {
    S Co = No / Nt, Cg = Ng / Nt;
    if (Co > 0)
      for (int a = 0; a < fl.ngO; ++a) e.N[fl.O[a]] = mole_fraction(N, nc, fl.O[a]) * Nop / Co;
    if (Cg > 0)
      for (int a = 0; a < fl.ngG; ++a) e.N[fl.G[a]] = mole_fraction(N, nc, fl.G[a]) * Ngp / Cg;
  };
  auto enthalpy = [&](S C, S dCdT, S xi, S dxidT, S dxidC, const DFunc& fn, PhaseT<S>& e) {
    S x[3] = {p, C, S(T)};
    S hbar = f_eval(fn, -1, x);
    if (hbar * xi < 0) atomicCAS(flag, 0, FL_ENTHALPY);
    e.h = hbar * xi;
    S dhbar_dT = f_eval(fn, 2, x);
    S dhbar_dC = 0;
    if (dCdT != 0) dhbar_dC = f_eval(fn, 1, x);
    e.dhdT = (dhbar_dT + dhbar_dC * dCdT) * xi + hbar * (dxidT + dxidC * dCdT);
  };
  if (NHC < 1e-300) {
    phase_clear(oil, nc);
    phase_clear(gas, nc);
    return;
  }
  S Cb = 0, Cd = 0;
  S Zo = No / NHC, Zg = Ng / NHC;
  if (Zg <= (Cb = f_eval(fl.bub, -1, pT))) {
    oil.present = true;
    phase_clear(gas, nc);
    inverse_group(No, Ng, oil);
    S Cgo = Ng / NHC;
    S x[3] = {p, Cgo, T};
    S xio = f_eval(fl.oden, -1, x);
    S Vo = (No + Ng) / xio;
    if (xio <= 0) atomicCAS(flag, 0, FL_DENSITY);
    oil.xi = xio;
    oil.V = Vo;
    S dxio_dp = f_eval(fl.oden, 0, x), dxio_dC = f_eval(fl.oden, 1, x), dxio_dT = f_eval(fl.oden, 2, x);
    S dCgo_dNo = -Cgo / NHC;
    S dCgo_dNg = (1 - Cgo) / NHC;
    S Vo_xio = Vo / xio;
    oil.dVdp = -Vo_xio * dxio_dp;
    oil.dVdT = -Vo_xio * dxio_dT;
    S dVodNo = (1 / xio) - Vo_xio * dxio_dC * dCgo_dNo;
    S dVodNg = (1 / xio) - Vo_xio * dxio_dC * dCgo_dNg;
    for (int a = 0; a < fl.ngO; ++a) oil.dVdN[fl.O[a]] = dVodNo;
    for (int a = 0; a < fl.ngG; ++a) oil.dVdN[fl.G[a]] = dVodNg;
    enthalpy(1, 0, xio, dxio_dT, dxio_dC, fl.oent, oil);
    oil.mu = f_eval(fl.ovis, -1, x);
  } else if (Zo <= (Cd = f_eval(fl.dew, -1, pT))) {
    phase_clear(oil, nc);
    gas.present = true;
    inverse_group(No, Ng, gas);
    S Cog = No / NHC;
    S x[3] = {p, Cog, T};
    S xig = f_eval(fl.gden, -1, x);
    S Vg = (No + Ng) / xig;
    if (xig <= 0) atomicCAS(flag, 0, FL_DENSITY);
    gas.xi = xig;
    gas.V = Vg;
    S dxig_dp = f_eval(fl.gden, 0, x), dxig_dC = f_eval(fl.gden, 1, x), dxig_dT = f_eval(fl.gden, 2, x);
    S dCgo_dNo = -(1 - Cog) / NHC;
    S dCgo_dNg = -Cog / NHC;
    S Vg_xig = Vg / xig;
    gas.dVdp = -Vg_xig * dxig_dp;
    gas.dVdT = -Vg_xig * dxig_dT;
    S dVgdNo = (1 / xig) - Vg_xig * dxig_dC * dCgo_dNo;
    S dVgdNg = (1 / xig) - Vg_xig * dxig_dC * dCgo_dNg;
    for (int a = 0; a < fl.ngO; ++a) gas.dVdN[fl.O[a]] = dVgdNo;
    for (int a = 0; a < fl.ngG; ++a) gas.dVdN[fl.G[a]] = dVgdNg;
    enthalpy(1, 0, xig, dxig_dT, dxig_dC, fl.gent, gas);
    gas.mu = f_eval(fl.gvis, -1, x);
  } else {
    oil.present = true;
    gas.present = true;
    S Cgo = Cb, Cog = Cd;
    S L = (Cog - Zo) / (Cog - (1 - Cgo));
    S Noo = L * NHC * (1 - Cgo);
    S Ngo = L * NHC * Cgo;
    S Nog = (1 - L) * NHC * Cog;
    S Ngg = (1 - L) * NHC * (1 - Cog);
    inverse_group(Noo, Ngo, oil);
    inverse_group(Nog, Ngg, gas);
    S xo[3] = {p, Cgo, T}, xg[3] = {p, Cog, T};
    S xio = f_eval(fl.oden, -1, xo);
    S xig = f_eval(fl.gden, -1, xg);
    S Vo = (Noo + Ngo) / xio;
    S Vg = (Nog + Ngg) / xig;
    oil.xi = xio;
    gas.xi = xig;
    oil.V = Vo;
    gas.V = Vg;
    S dCgo_dp = f_eval(fl.bub, 0, pT), dCog_dp = f_eval(fl.dew, 0, pT);
    S dCgo_dT = f_eval(fl.bub, 1, pT), dCog_dT = f_eval(fl.dew, 1, pT);
    S dLdp = (1 / (Cog - (1 - Cgo))) * ((1 - L) * dCog_dp - L * (dCgo_dp));
    S dLdT = (1 / (Cog - (1 - Cgo))) * ((1 - L) * dCog_dT - L * (dCgo_dT));
    S dLdNo = (1 / (Cog - (1 - Cgo))) * ((Zo - 1) / NHC);
    S dLdNg = (1 / (Cog - (1 - Cgo))) * (Zo / NHC);
    S dxio_dp = f_eval(fl.oden, 0, xo), dxio_dC = f_eval(fl.oden, 1, xo), dxio_dT = f_eval(fl.oden, 2, xo);
    S dxig_dp = f_eval(fl.gden, 0, xg), dxig_dC = f_eval(fl.gden, 1, xg), dxig_dT = f_eval(fl.gden, 2, xg);
    S dVodp = (Vo / L) * dLdp - (Vo / xio) * (dxio_dp + dxio_dC * dCgo_dp);
    S dVgdp = -(Vg / (1 - L)) * dLdp - (Vg / xig) * (dxig_dp + dxig_dC * dCog_dp);
    S dVodT = (Vo / L) * dLdT - (Vo / xio) * (dxio_dT + dxio_dC * dCgo_dT);
    S dVgdT = -(Vg / (1 - L)) * dLdT - (Vg / xig) * (dxig_dT + dxig_dC * dCog_dT);
    S dVodNo = (1 / xio) * (dLdNo * NHC + L);
    S dVodNg = (1 / xio) * (dLdNg * NHC + L);
    S dVgdNo = (1 / xig) * (-dLdNo * NHC + (1 - L));
    S dVgdNg = (1 / xig) * (-dLdNg * NHC + (1 - L));
    oil.dVdp = dVodp;
    oil.dVdT = dVodT;
    gas.dVdp = dVgdp;
    gas.dVdT = dVgdT;
    for (int a = 0; a < fl.ngO; ++a) {
      oil.dVdN[fl.O[a]] = dVodNo;
      gas.dVdN[fl.O[a]] = dVgdNo;
    }
    for (int a = 0; a < fl.ngG; ++a) {
      oil.dVdN[fl.G[a]] = dVodNg;
      gas.dVdN[fl.G[a]] = dVgdNg;
    }
    if (Cog - (1 - Cgo) > 0 || (1 - L) * dCog_dp - L * dCgo_dp > 0 || dVodp + dVgdp > 0 || dVodNo + dVgdNo <= 0 ||
        dVodNg + dVgdNg <= 0)
      atomicCAS(flag, 0, FL_BLACKOIL_CHECK);
    enthalpy(Cgo, dCgo_dT, xio, dxio_dT, dxio_dC, fl.oent, oil);
    enthalpy(Cog, dCog_dT, xig, dxig_dT, dxig_dC, fl.gent, gas);
    oil.mu = f_eval(fl.ovis, -1, xo);
    gas.mu = f_eval(fl.gvis, -1, xg);
  }
}

// Math.pow as HotSpot evaluates it for an exponent of exactly 2 (x * x);
// other exponents use CUDA's pow (within 2 ulp).
__device__ __forceinline__ double jpow(double x, double y) { return y == 2.0 ? x * x : pow(x, y); }
template <int K>
__device__ __forceinline__ Dual<K> jpow(const Dual<K>& x, double y) {
  return y == 2.0 ? x * x : dual_pow(x, y);
}

template <class S>
__device__ S eff_sat(const DCorey& c, int ph, S sat) {
  S Se = sat;
  Se -= c.Sr[ph];
  double denom = 1;
  for (int q = 0; q < 3; ++q) denom -= c.Sr[q];
  Se /= denom;
  return Se;
}

struct DCubic;
__device__ int cubic_phase_state(const DCubic& c, double p, double T, const double* Nin, Phase* ph, int* iters);

struct SimDev {
  int n, nc, nconn;
  const DCubic* cub;  // cubic equation of state (nullptr: black-oil)
  DFluid fl;
  DCorey co;
  int rf_kind;        // RSG_RF_*: Corey (co) or the tables below
  DFunc krw, krg, krow, krog, kro, pcow_t, pcgo_t;
  const double* phi0;
  const double* cr;
  const double* vol;
  const double* bf;  // body force per cell
  // primary
  double* p;
  double* p0;
  double* T;
  double* N;  // nc x n
  // phase records persisted between calls (nc x 3 x n for N and dVdN)
  double* phN;
  double* phdVdN;
  // secondaries
  double* S;       // 3 x n
  double* rho;     // 3 x n
  double* lambda;  // 3 x n
  double* Cxi;     // nc x 3 x n
  double* xi;      // 3 x n
  double* R;
  double* dRdp;
  double* dRdN;    // nc x n
  double* pcow;
  double* pcgo;
  int* present;    // bit mask per cell
  int* flag;
};

// Secondaries of one cell from its phase records: calculateFluidProperties,
// calculateRockProperties, CoreyRockFluid, calculateResidualVolume and the
// phase mobilities (field/CV.java:375-550).  S = double in the simulator; a
// dual number in the adjoint, which reads the same expressions' derivatives.
template <class S>
struct CellVals {
  S sat[3], rho[3], lambda[3], Cxi[NCM][3];
  S R, dRdp, dRdN[NCM], pcow, pcgo;
};

template <class S>
__device__ void cell_eval(const SimDev& d, int i, S p, double p0, const PhaseT<S>* ph, CellVals<S>& o) {
  const int nc = d.nc;
  const double V = d.vol[i];
  // calculateFluidProperties: rho = kg / V_l for present phases
  for (int a = 0; a < 3; ++a) {
    if (!ph[a].present) {
      o.rho[a] = S(0);
      continue;
    }
    S kg = 0;
    for (int nu = 0; nu < nc; ++nu) kg += d.fl.Mw[nu] * ph[a].N[nu];
    o.rho[a] = kg / ph[a].V;
  }
  // calculateRockProperties
  const double c = d.cr[i];
  const S dpp = p - p0;
  const S phi = d.phi0[i] * (1 + c * dpp + c * c * dpp * dpp / 2);
  S Vf = 0;
  for (int a = 0; a < 3; ++a) Vf += ph[a].V;
  for (int a = 0; a < 3; ++a) o.sat[a] = ph[a].V / Vf;
  // relative permeability and capillary pressures
  S kr[3];
  S pcow = 0, pcgo = 0;
  if (d.rf_kind == RSG_RF_TABULAR) {
    // TabularRockFluid.calculateRelativePermeability and capillary pressures
    // (rock/TabularRockFluid.java:60-91)
    kr[0] = f_eval(d.krw, -1, &o.sat[0]);
    kr[2] = f_eval(d.krg, -1, &o.sat[2]);
    if (o.sat[0] <= 0) atomicCAS(d.flag, 0, FL_NO_WATER);
    const S sow = o.sat[1] + o.sat[0];
    kr[1] = (o.sat[2] * f_eval(d.krog, -1, &sow) + o.sat[0] * f_eval(d.krow, -1, &o.sat[1])) / (o.sat[2] + o.sat[0]);
    pcow = f_eval(d.pcow_t, -1, &o.sat[0]);
    pcgo = f_eval(d.pcgo_t, -1, &o.sat[2]);
  } else if (d.rf_kind == RSG_RF_THREE_PHASE_TABULAR) {
    // ThreePhaseTabularRockFluid (rock/ThreePhaseTabularRockFluid.java:60-78)
    const S wg[2] = {o.sat[0], o.sat[2]};
    kr[0] = f_eval(d.krw, -1, wg);
    kr[2] = f_eval(d.krg, -1, wg);
    kr[1] = f_eval(d.kro, -1, wg);
    pcow = f_eval(d.pcow_t, -1, wg);
    pcgo = f_eval(d.pcgo_t, -1, wg);
  } else {
    // CoreyRockFluid
    for (int a = 0; a < 3; ++a) kr[a] = d.co.ke[a] * jpow(eff_sat(d.co, a, o.sat[a]), d.co.n[a]);
    S Sw = eff_sat(d.co, 0, o.sat[0]), So = eff_sat(d.co, 1, o.sat[1]);
    if (Sw > 0) pcow += d.co.cw / jpow(Sw, d.co.aw);
    if (So > 0) pcow -= d.co.cow / jpow(So, d.co.aow);
    S Sg = eff_sat(d.co, 2, o.sat[2]);
    if (Sg > 0) pcgo += d.co.cg / jpow(Sg, d.co.ag);
    if (So > 0) pcgo -= d.co.cog / jpow(So, d.co.aog);
  }
  o.pcow = pcow;
  o.pcgo = pcgo;
  // calculateResidualVolume
  S Vp = phi * V;
  S R = Vp;
  S dRdp = c * Vp;
  S dRdN[NCM];
  for (int nu = 0; nu < nc; ++nu) dRdN[nu] = S(0);
  for (int a = 0; a < 3; ++a) {
    R -= ph[a].V;
    dRdp -= ph[a].dVdp;
    for (int nu = 0; nu < nc; ++nu) dRdN[nu] -= ph[a].dVdN[nu];
  }
  o.R = R;
  o.dRdp = dRdp;
  for (int nu = 0; nu < nc; ++nu) o.dRdN[nu] = dRdN[nu];
  // mobilities and phase-component molar densities
  for (int a = 0; a < 3; ++a) {
    S lam = 0;
    if (ph[a].mu != 0) lam = kr[a] / ph[a].mu;
    o.lambda[a] = lam;
    for (int nu = 0; nu < nc; ++nu) o.Cxi[nu][a] = mole_fraction(ph[a].N, nc, nu) * ph[a].xi;
  }
}

// CV.calculateSecondaries on one cell; reads p, p0, T, N and the persisted
// phase records, writes all secondaries.
__device__ void cv_cell(const SimDev& d, int i, double p, double p0, double T, const double* N) {
  const int nc = d.nc, n = d.n;
  Phase ph[3];
  for (int a = 0; a < 3; ++a) {
    ph[a].present = (d.present[i] >> a) & 1;
    ph[a].V = ph[a].xi = ph[a].dVdp = ph[a].dVdT = ph[a].h = ph[a].dhdT = ph[a].mu = 0;
    for (int nu = 0; nu < nc; ++nu) {
      ph[a].N[nu] = d.phN[((int64_t)nu * 3 + a) * n + i];
      ph[a].dVdN[nu] = d.phdVdN[((int64_t)nu * 3 + a) * n + i];
    }
  }
  if (d.cub) {
    int it = 0;
    const int e = cubic_phase_state(*d.cub, p, T, N, ph, &it);
    if (e) atomicCAS(d.flag, 0, FL_CUBIC + e);
  } else {
    blackoil_state(d.fl, p, N, T, ph, d.flag);
  }
  CellVals<double> o;
  cell_eval(d, i, p, p0, ph, o);
  if (o.dRdp <= 0) atomicCAS(d.flag, 0, FL_DRDP);
  int mask = 0;
  for (int a = 0; a < 3; ++a) {
    d.S[(int64_t)a * n + i] = o.sat[a];
    d.rho[(int64_t)a * n + i] = o.rho[a];
    d.lambda[(int64_t)a * n + i] = o.lambda[a];
    d.xi[(int64_t)a * n + i] = ph[a].xi;
    for (int nu = 0; nu < nc; ++nu) {
      d.Cxi[((int64_t)nu * 3 + a) * n + i] = o.Cxi[nu][a];
      d.phN[((int64_t)nu * 3 + a) * n + i] = ph[a].N[nu];
      d.phdVdN[((int64_t)nu * 3 + a) * n + i] = ph[a].dVdN[nu];
    }
    if (ph[a].present) mask |= 1 << a;
  }
  d.present[i] = mask;
  d.R[i] = o.R;
  d.dRdp[i] = o.dRdp;
  for (int nu = 0; nu < nc; ++nu) d.dRdN[(int64_t)nu * n + i] = o.dRdN[nu];
  d.pcow[i] = o.pcow;
  d.pcgo[i] = o.pcgo;
}

__global__ void k_cv(SimDev d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  double N[NCM];
  for (int nu = 0; nu < d.nc; ++nu) N[nu] = d.N[(int64_t)nu * d.n + i];
  cv_cell(d, i, d.p[i], d.p0[i], d.T[i], N);
}

__device__ __forceinline__ double phase_pressure(const SimDev& d, int e, int ph) {
  double p = d.p[e];
  return ph == 0 ? p - d.pcow[e] : (ph == 1 ? p : p + d.pcgo[e]);
}

struct ConnDev {
  const int* conn;
  const int* md_ptr;
  const int* md_el;
  const double* md_k;
  double* rho_cs;  // 3 x nconn
  double* u;       // 3 x nconn
  int* up;         // 3 x nconn
};

// CS.calculateSecondaries (field/CS.java:94-155)
__global__ void k_cs(SimDev d, ConnDev c) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nconn) return;
  const int h = c.conn[2 * q], t = c.conn[2 * q + 1];
  const int nc_ = d.nconn;
  double rho[3];
  for (int a = 0; a < 3; ++a) {
    rho[a] = 0;
    double Sh = d.S[(int64_t)a * d.n + h], St = d.S[(int64_t)a * d.n + t];
    double S = Sh + St;
    double av = (Sh * d.rho[(int64_t)a * d.n + h] + St * d.rho[(int64_t)a * d.n + t]) / S;
    if (!isnan(av)) rho[a] = av;
    c.rho_cs[(int64_t)a * nc_ + q] = rho[a];
  }
  for (int a = 0; a < 3; ++a) {
    double D = 0;
    for (int m = c.md_ptr[q]; m < c.md_ptr[q + 1]; ++m) {
      int ek = c.md_el[m];
      double psi = phase_pressure(d, ek, a) + rho[a] * d.bf[ek];
      D += c.md_k[m] * psi;
    }
    int up = (D > 0) ? h : t;
    c.up[(int64_t)a * nc_ + q] = up;
    c.u[(int64_t)a * nc_ + q] = d.lambda[(int64_t)a * d.n + up] * D;
  }
}

// assemblePressureJacobianFlux per connection (Discretisation.java:459-561)
__global__ void k_flux_conn(SimDev d, ConnDev c, double* Jh, double* Jt, double* rh, double* rt) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nconn) return;
  const int i = c.conn[2 * q], j = c.conn[2 * q + 1];
  const int n = d.n, nc = d.nc, ncn = d.nconn;
  double dRh[NCM], dRt[NCM];
  for (int nu = 0; nu < nc; ++nu) {
    dRh[nu] = d.dRdN[(int64_t)nu * n + i];
    dRt[nu] = d.dRdN[(int64_t)nu * n + j];
  }
  int up[3];
  bool pres[3];
  double rho[3];
  for (int a = 0; a < 3; ++a) {
    up[a] = c.up[(int64_t)a * ncn + q];
    pres[a] = (d.present[up[a]] >> a) & 1;
    rho[a] = c.rho_cs[(int64_t)a * ncn + q];
  }
  double ri = 0, rj = 0;
  for (int m = c.md_ptr[q]; m < c.md_ptr[q + 1]; ++m) {
    const int ik = c.md_el[m];
    const double tk = c.md_k[m];
    const double b = d.bf[ik];
    double Ji = 0, Jj = 0;
    for (int a = 0; a < 3; ++a) {
      if (!pres[a]) continue;
      double psi = phase_pressure(d, ik, a) + rho[a] * b;
      const double lam = d.lambda[(int64_t)a * n + up[a]];
      for (int nu = 0; nu < nc; ++nu) {
        double phaseCompMob = d.Cxi[((int64_t)nu * 3 + a) * n + up[a]] * lam;
        double dNdt = -phaseCompMob * tk * psi;
        double d2Ndtp = -phaseCompMob * tk;
        ri += dRh[nu] * dNdt;
        rj += -dRt[nu] * dNdt;
        Ji += dRh[nu] * d2Ndtp;
        Jj += -dRt[nu] * d2Ndtp;
      }
    }
    Jh[m] = Ji;
    Jt[m] = Jj;
  }
  rh[q] = ri;
  rt[q] = rj;
}

// The same assembly with each block's interaction-region stencils (the MD
// lists of its 128 connections: element indices and transmissibilities,
// contiguous in memory) staged into shared memory by TMA: one thread arms an
// mbarrier and issues 1D tensor copies of 256 entries (cp.async.bulk.tensor,
// box 256, x aligned to 16 bytes, the part past the array filled with
// zeros); the block's Jacobian contributions are written back from shared
// memory with coalesced stores.  Arithmetic and order as k_flux_conn, so the
// results are identical.
constexpr int FLUX_BLOCK = 128;
constexpr int TMA_BOX = 256;

__device__ __forceinline__ void tma_load_1d(unsigned dst, const CUtensorMap* map, int x, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(bar)
      : "memory");
}

__device__ __forceinline__ bool tma_wait(unsigned bar, unsigned parity) {
  for (int i = 0; i < (1 << 22); ++i) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__global__ void __launch_bounds__(FLUX_BLOCK) k_flux_conn_tma(SimDev d, ConnDev c, double* Jh, double* Jt, double* rh,
                                                             double* rt, const __grid_constant__ CUtensorMap tm_el,
                                                             const __grid_constant__ CUtensorMap tm_k, int chunks) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bar;
  int* s_el = reinterpret_cast<int*>(sm);
  double* s_k = reinterpret_cast<double*>(sm + (size_t)chunks * TMA_BOX * sizeof(int));
  double* s_jh = s_k + (size_t)chunks * TMA_BOX;
  double* s_jt = s_jh + (size_t)chunks * TMA_BOX;
  const int q0 = blockIdx.x * FLUX_BLOCK, q1 = min(q0 + FLUX_BLOCK, d.nconn);
  const int m0 = c.md_ptr[q0], m1 = c.md_ptr[q1];
  const int e0 = m0 & ~3, k0 = m0 & ~1;  // 16-byte aligned starts
  const int ce = (m1 - e0 + TMA_BOX - 1) / TMA_BOX, ck = (m1 - k0 + TMA_BOX - 1) / TMA_BOX;
  const unsigned b = (unsigned)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    // the barrier's initialisation is visible to the tensor copies
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
                 "r"((unsigned)(ce * TMA_BOX * sizeof(int) + ck * TMA_BOX * sizeof(double)))
                 : "memory");
    for (int q = 0; q < ce; ++q)
      tma_load_1d((unsigned)__cvta_generic_to_shared(s_el + q * TMA_BOX), &tm_el, e0 + q * TMA_BOX, b);
    for (int q = 0; q < ck; ++q)
      tma_load_1d((unsigned)__cvta_generic_to_shared(s_k + q * TMA_BOX), &tm_k, k0 + q * TMA_BOX, b);
  }
  __syncthreads();
  if (!__syncthreads_and(tma_wait(b, 0))) {
    // the copies did not land in time: give them time to end, report, stop
    if (threadIdx.x == 0) {
      tma_wait(b, 0);
      atomicCAS(d.flag, 0, FL_TMA);
    }
    return;
  }
  const int q = q0 + threadIdx.x;
  if (q < q1) {
    const int i = c.conn[2 * q], j = c.conn[2 * q + 1];
    const int n = d.n, nc = d.nc, ncn = d.nconn;
    double dRh[NCM], dRt[NCM];
    for (int nu = 0; nu < nc; ++nu) {
      dRh[nu] = d.dRdN[(int64_t)nu * n + i];
      dRt[nu] = d.dRdN[(int64_t)nu * n + j];
    }
    int up[3];
    bool pres[3];
    double rho[3];
    for (int a = 0; a < 3; ++a) {
      up[a] = c.up[(int64_t)a * ncn + q];
      pres[a] = (d.present[up[a]] >> a) & 1;
      rho[a] = c.rho_cs[(int64_t)a * ncn + q];
    }
    double ri = 0, rj = 0;
    for (int m = c.md_ptr[q]; m < c.md_ptr[q + 1]; ++m) {
      const int ik = s_el[m - e0];
      const double tk = s_k[m - k0];
      const double bfk = d.bf[ik];
      double Ji = 0, Jj = 0;
      for (int a = 0; a < 3; ++a) {
        if (!pres[a]) continue;
        double psi = phase_pressure(d, ik, a) + rho[a] * bfk;
        const double lam = d.lambda[(int64_t)a * n + up[a]];
        for (int nu = 0; nu < nc; ++nu) {
          double phaseCompMob = d.Cxi[((int64_t)nu * 3 + a) * n + up[a]] * lam;
          double dNdt = -phaseCompMob * tk * psi;
          double d2Ndtp = -phaseCompMob * tk;
          ri += dRh[nu] * dNdt;
          rj += -dRt[nu] * dNdt;
          Ji += dRh[nu] * d2Ndtp;
          Jj += -dRt[nu] * d2Ndtp;
        }
      }
      s_jh[m - k0] = Ji;
      s_jt[m - k0] = Jj;
    }
    rh[q] = ri;
    rt[q] = rj;
  }
  __syncthreads();
  for (int m = m0 + threadIdx.x; m < m1; m += FLUX_BLOCK) {
    Jh[m] = s_jh[m - k0];
    Jt[m] = s_jt[m - k0];
  }
}

struct AsmDev {
  const int* cc;      // incident connections (2c + side), 6 per cell
  const int* ccount;
  const int* md_ptr;
  const int* pos_here;
  const int* pos_there;
  const int* rowptr;
  const int* diag;
  const int* src_ptr;  // regular sources per cell
  const int* src_id;
  const double* src_q;  // nsrc x NCM
  const int* locked;
  const double* p_prev;
  const double* R_prev;
};

// Row gather of the Jacobian and residual, then LinearSolver.solve's
// sign change and locked rows (numerics/LinearSolver.java:246-260).
__global__ void k_assemble_rows(SimDev d, AsmDev a, const double* Jh, const double* Jt, const double* rh,
                                const double* rt, double dt, double* val, double* b, double* rawJ, double* rawB) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int r0 = a.rowptr[e], r1 = a.rowptr[e + 1];
  for (int q = r0; q < r1; ++q) val[q] = 0;
  double be = 0;
  for (int k = 0; k < a.ccount[e]; ++k) {
    const int code = a.cc[(int64_t)e * 6 + k];
    const int c = code >> 1;
    const bool here = !(code & 1);
    if (here) {
      for (int m = a.md_ptr[c]; m < a.md_ptr[c + 1]; ++m) {
        const int pos = a.pos_here[m];
        if (pos >= r0 && pos < r1) val[pos] += Jh[m];
        else atomicCAS(d.flag, 0, FL_PATTERN);
      }
      be += rh[c];
    } else {
      for (int m = a.md_ptr[c]; m < a.md_ptr[c + 1]; ++m) {
        const int pos = a.pos_there[m];
        if (pos >= r0 && pos < r1) val[pos] += Jt[m];
        else atomicCAS(d.flag, 0, FL_PATTERN);
      }
      be += rt[c];
    }
  }
  // assemblePressureJacobianDiagonal
  const double dpp = d.p[e] - a.p_prev[e];
  const double dRdp = d.dRdp[e];
  be += (a.R_prev[e] + dRdp * dpp) / dt;
  val[a.diag[e]] += dRdp / dt;
  // assemblePressureRegularSource
  for (int s = a.src_ptr[e]; s < a.src_ptr[e + 1]; ++s) {
    const double* q = a.src_q + (int64_t)a.src_id[s] * NCM;
    for (int nu = 0; nu < d.nc; ++nu) be += d.dRdN[(int64_t)nu * d.n + e] * q[nu];
  }
  if (rawJ) {
    for (int q = r0; q < r1; ++q) rawJ[q] = val[q];
  }
  be *= -1;
  if (rawB) rawB[e] = be;
  if (a.locked[e]) {
    for (int q = r0; q < r1; ++q) val[q] = (q == a.diag[e]) ? 1.0 : 0.0;
    be = 0;
  }
  b[e] = be;
}

// PressureNewtonRaphson.updatePressure (:340-359): p += dp, max |dp/p_prev|
__global__ void k_update_pressure(SimDev d, double* dp, const int* locked, const double* p_prev,
                                  unsigned long long* dpmax_bits, int* bad_row, double* dp0) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  if (locked[i]) dp[i] = 0;  // LinearSolver.solve: x[locked] = 0
  double dpi = dp[i];
  double pn = d.p[i] + dpi;
  if (pn <= 0) atomicMin(bad_row, i + 1);
  d.p[i] = pn;
  double r = fabs(dpi / p_prev[i]);
  atomicMax(dpmax_bits, (unsigned long long)__double_as_longlong(r));
  if (i == 0) *dp0 = dpi;
}

// MolarMassExplicit.calculateMolarMassFlux per connection
__global__ void k_molar_conn(SimDev d, ConnDev c, double* cf) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nconn) return;
  const int n = d.n, nc = d.nc, ncn = d.nconn;
  double flux[NCM];
  for (int nu = 0; nu < nc; ++nu) flux[nu] = 0;
  for (int a = 0; a < 3; ++a) {
    int up = c.up[(int64_t)a * ncn + q];
    if (!((d.present[up] >> a) & 1)) continue;
    double D = c.u[(int64_t)a * ncn + q];
    for (int nu = 0; nu < nc; ++nu) flux[nu] += d.Cxi[((int64_t)nu * 3 + a) * n + up] * D;
  }
  for (int nu = 0; nu < nc; ++nu) cf[(int64_t)nu * ncn + q] = flux[nu];
}

// dN gather, sources, locks, update with the negative-moles test
__global__ void k_molar_cells(SimDev d, AsmDev a, const double* cf, double dt, const double* N_prev, int truncate,
                              int* bad_row, double* dN_out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int n = d.n, nc = d.nc, ncn = d.nconn;
  double dN[NCM];
  for (int nu = 0; nu < nc; ++nu) dN[nu] = 0;
  for (int k = 0; k < a.ccount[e]; ++k) {
    const int code = a.cc[(int64_t)e * 6 + k];
    const int c = code >> 1;
    const bool here = !(code & 1);
    for (int nu = 0; nu < nc; ++nu) {
      double f = cf[(int64_t)nu * ncn + c];
      if (here) dN[nu] -= dt * f;
      else dN[nu] += dt * f;
    }
  }
  for (int s = a.src_ptr[e]; s < a.src_ptr[e + 1]; ++s) {
    const double* q = a.src_q + (int64_t)a.src_id[s] * NCM;
    for (int nu = 0; nu < nc; ++nu) dN[nu] += dt * q[nu];
  }
  for (int nu = 0; nu < nc; ++nu) dN_out[(int64_t)nu * n + e] = dN[nu];
  if (a.locked[e])
    for (int nu = 0; nu < nc; ++nu) dN[nu] = 0;
  for (int nu = 0; nu < nc; ++nu) {
    double Nold = N_prev[(int64_t)nu * n + e];
    double Nnew = Nold + dN[nu];
    if (Nnew < 0) {
      if (truncate) Nnew = 0;
      else atomicMin(bad_row, e + 1);
    }
    d.N[(int64_t)nu * n + e] = Nnew;
  }
}

// Field.volumeBalance (field/Field.java:390-447) per cell
struct InitDev {
  double datum_depth, datum_pressure;
  DFunc temperature;
  DFunc frac[NCM];
  const double* zc;     // cell centre z
  const int* fixed_id;  // fixed source per cell (-1 none); the last one listed wins
  const double* fixed_T;
  const double* fixed_C;  // nsrc x NCM, normalised
};

__device__ void volume_balance(const SimDev& d, const InitDev& in, int i, const double* C, double p, double T) {
  const int nc = d.nc, n = d.n;
  double N[NCM];
  for (int nu = 0; nu < nc; ++nu) N[nu] = 1 * C[nu];
  double dz = in.zc[i] - in.datum_depth;
  double p0 = p;
  cv_cell(d, i, p, p0, T, N);
  int iters = 0;
  do {
    double dRdNt = 0;
    for (int nu = 0; nu < nc; ++nu) dRdNt += d.dRdN[(int64_t)nu * n + i] * C[nu];
    if (dRdNt == 0) {
      atomicCAS(d.flag, 0, FL_DRDP);
      return;
    }
    double Nt = 0;
    for (int nu = 0; nu < nc; ++nu) Nt += N[nu];
    double dNt = -d.R[i] / dRdNt;
    double alpha = 1;
    for (int h = 0; h < 2100 && Nt + alpha * dNt < 0; ++h) alpha /= 2;
    Nt += alpha * dNt;
    for (int nu = 0; nu < nc; ++nu) N[nu] = Nt * C[nu];
    double pp = in.datum_pressure;
    for (int a = 0; a < 3; ++a) pp -= G_ACC * d.rho[(int64_t)a * n + i] * d.S[(int64_t)a * n + i] * dz;
    p = pp;
    p0 = pp;
    cv_cell(d, i, p, p0, T, N);
    iters++;
  } while (iters < 3 || (fabs(d.R[i]) > 1.0e-9 && iters < 50));
  d.p[i] = p;
  d.p0[i] = p0;
  d.T[i] = T;
  for (int nu = 0; nu < nc; ++nu) d.N[(int64_t)nu * n + i] = N[nu];
}

__global__ void k_init(SimDev d, InitDev in) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const int nc = d.nc;
  double z = in.zc[i];
  double C[NCM];
  double sum = 0;
  double T = f_eval(in.temperature, -1, &z);
  for (int nu = 0; nu < nc; ++nu) {
    C[nu] = f_eval(in.frac[nu], -1, &z);
    sum += C[nu];
  }
  if (sum == 0) {
    C[0] = 1;
    sum = 1;
  }
  for (int nu = 0; nu < nc; ++nu) C[nu] /= sum;
  volume_balance(d, in, i, C, in.datum_pressure, T);
  int f = in.fixed_id[i];
  if (f >= 0) {
    double Cf[NCM];
    for (int nu = 0; nu < nc; ++nu) Cf[nu] = in.fixed_C[(int64_t)f * NCM + nu];
    volume_balance(d, in, i, Cf, in.datum_pressure, in.fixed_T[f]);
  }
}

__global__ void k_copy(int64_t n, const double* __restrict__ a, double* __restrict__ b) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

__global__ void k_zero(int64_t n, double* __restrict__ a) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = 0;
}

// deterministic per-block partial sums of dN (mass balance diagnostic)
__global__ void k_sum_blocks(int64_t n, const double* __restrict__ a, double* part) {
  __shared__ double sh[256];
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) s += a[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

#include "cubic.cuh"

// ------------------------------------------------------------ adjoint ----
// Reverse-mode sensitivities of the sequential pressure / explicit-moles step
// with respect to per-element log-permeability (no reference counterpart).
// Per step n, with x_e = (p_e, N_e,0..N_e,nc-1) evaluated at (p^{n+1}, N^n):
//   F_e = sum_nu dRdN_e,nu Q_e,nu + (R(p^n, N^n)_e + dRdp_e (p^{n+1}_e - p^n_e)) / dt
//   Q_e,nu = sum_c s_ec cf_c,nu + q_e,nu     (net molar inflow, s = -1 here, +1 there)
//   cf_c,nu = sum_a [present] Cxi_up,nu,a lambda_up,a D_c,a,
//   D_c,a = sum_m t_cm (p_m + pc_m,a + rho_cs,a bf_m)
// (Discretisation.java:365-561 and 769-919).  The pressure step solves F = 0
// (locked rows: p = p^n), and N^{n+1} = N^n + dt Q off the locked cells.
// Local derivatives of every cell quantity come from the dual-number
// evaluation of the same property chain; connection terms are
// differentiated by hand below.
constexpr int ADJ_NC = 3;          // components the adjoint supports
constexpr int ADJ_K = 1 + ADJ_NC;  // unknowns per cell: p and the moles
using AD = Dual<ADJ_K>;

// derivative records: quantity q, unknown k of cell i at rec[(q * K + k) * n + i]
enum { Q_SAT = 0, Q_RHO = 3, Q_LAM = 6, Q_PCOW = 9, Q_PCGO = 10, Q_R = 11, Q_DRDP = 12, Q_DRDN = 13 };
__host__ __device__ inline int q_cxi(int nc, int nu, int a) { return Q_DRDN + nc + nu * 3 + a; }
__host__ __device__ inline int adj_nq(int nc) { return Q_DRDN + 4 * nc; }

struct Rec {
  const double* r;
  int n, K;
  __device__ double operator()(int q, int k, int i) const { return r[((int64_t)q * K + k) * n + i]; }
};

// Dual-number evaluation of the property chain of every cell at (p, N); the
// persisted phase records enter as constants as they do in cv_cell.
__global__ void __launch_bounds__(128) k_cell_dual(SimDev d, const double* __restrict__ pv,
                                                   const double* __restrict__ Nv, double* __restrict__ rec) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const int nc = d.nc, n = d.n, K = 1 + nc;
  PhaseT<AD> ph[3];
  for (int a = 0; a < 3; ++a) {
    ph[a].present = (d.present[i] >> a) & 1;
    ph[a].V = ph[a].xi = ph[a].dVdp = ph[a].dVdT = ph[a].h = ph[a].dhdT = ph[a].mu = AD(0);
    for (int nu = 0; nu < nc; ++nu) {
      ph[a].N[nu] = AD(d.phN[((int64_t)nu * 3 + a) * n + i]);
      ph[a].dVdN[nu] = AD(d.phdVdN[((int64_t)nu * 3 + a) * n + i]);
    }
  }
  AD p = AD::var(pv[i], 0);
  AD N[NCM];
  for (int nu = 0; nu < nc; ++nu) N[nu] = AD::var(Nv[(int64_t)nu * n + i], 1 + nu);
  blackoil_state(d.fl, p, N, d.T[i], ph, d.flag);
  CellVals<AD> o;
  cell_eval(d, i, p, d.p0[i], ph, o);
  auto put = [&](int q, const AD& x) {
    for (int k = 0; k < K; ++k) rec[((int64_t)q * K + k) * n + i] = x.d[k];
  };
  for (int a = 0; a < 3; ++a) {
    put(Q_SAT + a, o.sat[a]);
    put(Q_RHO + a, o.rho[a]);
    put(Q_LAM + a, o.lambda[a]);
    for (int nu = 0; nu < nc; ++nu) put(q_cxi(nc, nu, a), o.Cxi[nu][a]);
  }
  put(Q_PCOW, o.pcow);
  put(Q_PCGO, o.pcgo);
  put(Q_R, o.R);
  put(Q_DRDP, o.dRdp);
  for (int nu = 0; nu < nc; ++nu) put(Q_DRDN + nu, o.dRdN[nu]);
}

// d(phase pressure of phase a at cell e)/dx_k
__device__ __forceinline__ double dpp_dx(const Rec& r, int e, int a, int k) {
  const double dp = k == 0 ? 1.0 : 0.0;
  return a == 0 ? dp - r(Q_PCOW, k, e) : (a == 1 ? dp : dp + r(Q_PCGO, k, e));
}

struct AdjConn {
  const int* md_ptr;
  const int* md_el;
  const double* md_k;
  const int* conn;
  const double* rho_cs;
  const int* up;
};

// Derivatives of w . cf_c for one connection, w a weight per component:
// fills, per MD entry m of c and unknown k, the derivative with respect to
// x_k of cell el_m (to the slots of the here / there cells also go the
// density-average and upwind terms), and the theta-pair weights
// mu_a = [present] lambda_up,a sum_nu w_nu Cxi_up,nu,a  and
// mu_3 = sum_a mu_a rho_cs,a (potentials p + pc_a and bf).
__device__ void conn_vjp(const SimDev& d, const AdjConn& c, const Rec& r, int q, const double* w, int kmax,
                         double (*out)[ADJ_K], double* mu) {
  const int n = d.n, nc = d.nc, ncn = d.nconn;
  const int h = c.conn[2 * q], t = c.conn[2 * q + 1];
  const int m0 = c.md_ptr[q], m1 = c.md_ptr[q + 1];
  for (int m = 0; m < m1 - m0; ++m)
    for (int k = 0; k < kmax; ++k) out[m][k] = 0;
  int mh = -1, mt = -1;
  double B = 0;
  for (int m = m0; m < m1; ++m) {
    const int e = c.md_el[m];
    if (e == h) mh = m - m0;
    if (e == t) mt = m - m0;
    B += c.md_k[m] * d.bf[e];
  }
  double mu3 = 0;
  for (int a = 0; a < 3; ++a) {
    const int up = c.up[(int64_t)a * ncn + q];
    const bool pres = (d.present[up] >> a) & 1;
    const double rcs = c.rho_cs[(int64_t)a * ncn + q];
    const double lam = d.lambda[(int64_t)a * n + up];
    double Mc = 0;
    if (pres)
      for (int nu = 0; nu < nc; ++nu) Mc += w[nu] * d.Cxi[((int64_t)nu * 3 + a) * n + up];
    Mc *= pres ? lam : 0.0;
    mu[a] = Mc;
    mu3 += Mc * rcs;
    if (!pres) continue;
    // D_c,a and the phase-pressure terms
    double D = 0;
    for (int m = m0; m < m1; ++m) {
      const int e = c.md_el[m];
      const double pp = a == 0 ? d.p[e] - d.pcow[e] : (a == 1 ? d.p[e] : d.p[e] + d.pcgo[e]);
      D += c.md_k[m] * (pp + rcs * d.bf[e]);
      for (int k = 0; k < kmax; ++k) out[m - m0][k] += Mc * c.md_k[m] * dpp_dx(r, e, a, k);
    }
    // upwind cell: d(Cxi lambda)/dx
    const int mu_slot = up == h ? mh : mt;
    if (mu_slot >= 0)
      for (int k = 0; k < kmax; ++k) {
        double s = 0;
        for (int nu = 0; nu < nc; ++nu)
          s += w[nu] * (r(q_cxi(nc, nu, a), k, up) * lam + d.Cxi[((int64_t)nu * 3 + a) * n + up] * r(Q_LAM + a, k, up));
        out[mu_slot][k] += D * s;
      }
    // density average: d rho_cs / dx_h and dx_t
    const double Sh = d.S[(int64_t)a * n + h], St = d.S[(int64_t)a * n + t];
    const double Ssum = Sh + St;
    if (Ssum != 0 && !isnan(rcs) && Mc * B != 0) {
      const double rh = d.rho[(int64_t)a * n + h], rt = d.rho[(int64_t)a * n + t];
      for (int k = 0; k < kmax; ++k) {
        const double gh = (r(Q_SAT + a, k, h) * (rh - rcs) + Sh * r(Q_RHO + a, k, h)) / Ssum;
        const double gt = (r(Q_SAT + a, k, t) * (rt - rcs) + St * r(Q_RHO + a, k, t)) / Ssum;
        if (mh >= 0) out[mh][k] += Mc * B * gh;
        if (mt >= 0) out[mt][k] += Mc * B * gt;
      }
    }
  }
  mu[3] = mu3;
}

constexpr int ADJ_MAXMD = 32;

// Exact pressure Jacobian of the connection terms: rows here (weights
// -dRdN_here) and there (+dRdN_there), columns the MD cells.
__global__ void __launch_bounds__(128) k_adj_conn_jac(SimDev d, AdjConn c, Rec r, double* __restrict__ Jh,
                                                      double* __restrict__ Jt, int* flag) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nconn) return;
  const int n = d.n, nc = d.nc;
  const int h = c.conn[2 * q], t = c.conn[2 * q + 1];
  const int m0 = c.md_ptr[q], m1 = c.md_ptr[q + 1];
  if (m1 - m0 > ADJ_MAXMD) {
    atomicCAS(flag, 0, 1);
    return;
  }
  double out[ADJ_MAXMD][ADJ_K], mu[4], w[NCM];
  for (int nu = 0; nu < nc; ++nu) w[nu] = -d.dRdN[(int64_t)nu * n + h];
  conn_vjp(d, c, r, q, w, 1, out, mu);
  for (int m = m0; m < m1; ++m) Jh[m] = out[m - m0][0];
  for (int nu = 0; nu < nc; ++nu) w[nu] = d.dRdN[(int64_t)nu * n + t];
  conn_vjp(d, c, r, q, w, 1, out, mu);
  for (int m = m0; m < m1; ++m) Jt[m] = out[m - m0][0];
}

// Vector-Jacobian product of sum_e z_e . Q_e for weights z (nc x n): per MD
// entry the K derivatives (cmd, entry-major) and the theta-pair weights.
__global__ void __launch_bounds__(128) k_adj_conn_vjp(SimDev d, AdjConn c, Rec r, const double* __restrict__ z,
                                                      double* __restrict__ cmd, double* __restrict__ mu, int* flag) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= d.nconn) return;
  const int n = d.n, nc = d.nc, K = 1 + nc, ncn = d.nconn;
  const int h = c.conn[2 * q], t = c.conn[2 * q + 1];
  const int m0 = c.md_ptr[q], m1 = c.md_ptr[q + 1];
  if (m1 - m0 > ADJ_MAXMD) {
    atomicCAS(flag, 0, 1);
    return;
  }
  double out[ADJ_MAXMD][ADJ_K], mq[4], w[NCM];
  for (int nu = 0; nu < nc; ++nu) w[nu] = z[(int64_t)nu * n + t] - z[(int64_t)nu * n + h];
  conn_vjp(d, c, r, q, w, K, out, mq);
  for (int m = m0; m < m1; ++m)
    for (int k = 0; k < K; ++k) cmd[(int64_t)m * K + k] = out[m - m0][k];
  for (int a = 0; a < 4; ++a) mu[(int64_t)a * ncn + q] = mq[a];
}

// Per cell: the sum of its MD-entry derivatives (ascending entry order).
__global__ void k_adj_gather(int n, int K, const int* __restrict__ inv_ptr, const int* __restrict__ inv_q,
                             const double* __restrict__ cmd, double* __restrict__ g) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s[ADJ_K];
  for (int k = 0; k < K; ++k) s[k] = 0;
  for (int j = inv_ptr[e]; j < inv_ptr[e + 1]; ++j) {
    const int64_t m = inv_q[j];
    for (int k = 0; k < K; ++k) s[k] += cmd[m * K + k];
  }
  for (int k = 0; k < K; ++k) g[(int64_t)k * n + e] = s[k];
}

// Net molar inflow Q (no dt) in the order k_molar_cells accumulates dN.
__global__ void k_adj_inflow(SimDev d, AsmDev a, const double* __restrict__ cf, double* __restrict__ Q) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int n = d.n, nc = d.nc, ncn = d.nconn;
  double s[NCM];
  for (int nu = 0; nu < nc; ++nu) s[nu] = 0;
  for (int k = 0; k < a.ccount[e]; ++k) {
    const int code = a.cc[(int64_t)e * 6 + k];
    const int c = code >> 1;
    const bool here = !(code & 1);
    for (int nu = 0; nu < nc; ++nu) s[nu] += here ? -cf[(int64_t)nu * ncn + c] : cf[(int64_t)nu * ncn + c];
  }
  for (int j = a.src_ptr[e]; j < a.src_ptr[e + 1]; ++j) {
    const double* qs = a.src_q + (int64_t)a.src_id[j] * NCM;
    for (int nu = 0; nu < nc; ++nu) s[nu] += qs[nu];
  }
  for (int nu = 0; nu < nc; ++nu) Q[(int64_t)nu * n + e] = s[nu];
}

// Exact pressure Jacobian rows: connection terms gathered as
// k_assemble_rows gathers the Newton Jacobian, plus the cell's own
// derivatives of dRdN and dRdp; locked rows are identity rows.
__global__ void k_adj_rows(SimDev d, AsmDev a, Rec r, const double* __restrict__ Jh, const double* __restrict__ Jt,
                           const double* __restrict__ Q, const double* __restrict__ p_prev, double dt,
                           double* __restrict__ val) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int n = d.n, nc = d.nc;
  const int r0 = a.rowptr[e], r1 = a.rowptr[e + 1];
  for (int q = r0; q < r1; ++q) val[q] = 0;
  if (a.locked[e]) {
    val[a.diag[e]] = 1.0;
    return;
  }
  for (int k = 0; k < a.ccount[e]; ++k) {
    const int code = a.cc[(int64_t)e * 6 + k];
    const int c = code >> 1;
    const bool here = !(code & 1);
    for (int m = a.md_ptr[c]; m < a.md_ptr[c + 1]; ++m) {
      const int pos = here ? a.pos_here[m] : a.pos_there[m];
      if (pos >= r0 && pos < r1) val[pos] += here ? Jh[m] : Jt[m];
      else atomicCAS(d.flag, 0, FL_PATTERN);
    }
  }
  double diag = d.dRdp[e] / dt + (d.p[e] - p_prev[e]) / dt * r(Q_DRDP, 0, e);
  for (int nu = 0; nu < nc; ++nu) diag += Q[(int64_t)nu * n + e] * r(Q_DRDN + nu, 0, e);
  val[a.diag[e]] += diag;
}

// Weights on Q: z = dt (aN off the locked cells + objective weights) - y dRdN
__global__ void k_adj_z(int n, int nc, const int* __restrict__ locked, const double* __restrict__ objw,
                        const double* __restrict__ cw, const double* __restrict__ aN, const double* __restrict__ y,
                        const double* __restrict__ dRdN, double dt, double* __restrict__ z) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const bool lk = locked[e];
  for (int nu = 0; nu < nc; ++nu) {
    double w = (lk ? 0.0 : aN[(int64_t)nu * n + e]) + objw[e] * cw[nu];
    double v = dt * w;
    if (y && !lk) v -= y[e] * dRdN[(int64_t)nu * n + e];
    z[(int64_t)nu * n + e] = v;
  }
}

__global__ void k_adj_rhs(int n, const double* __restrict__ aP, const double* __restrict__ g0, double* __restrict__ w) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) w[e] = aP[e] + g0[e];
}

// Potentials of the theta pairs: p + pc for each phase, and the body force
__global__ void k_adj_phi(SimDev d, double* __restrict__ phi) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int n = d.n;
  phi[e] = d.p[e] - d.pcow[e];
  phi[n + e] = d.p[e];
  phi[2 * (int64_t)n + e] = d.p[e] + d.pcgo[e];
  phi[3 * (int64_t)n + e] = d.bf[e];
}

// Adjoint state of step n from that of step n+1 (g: VJP of z^M - z^F)
__global__ void k_adj_update(SimDev d, const int* __restrict__ locked, Rec ra, Rec rb, const double* __restrict__ y,
                             const double* __restrict__ g, const double* __restrict__ Q,
                             const double* __restrict__ p_prev, double dt, double* __restrict__ aP,
                             double* __restrict__ aN) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.n) return;
  const int n = d.n, nc = d.nc;
  const bool lk = locked[e];
  const double yt = lk ? 0.0 : y[e];
  const double dpp = d.p[e] - p_prev[e];
  for (int nu = 0; nu < nc; ++nu) {
    const int k = 1 + nu;
    double diag = dpp / dt * ra(Q_DRDP, k, e) + rb(Q_R, k, e) / dt;
    for (int mu = 0; mu < nc; ++mu) diag += Q[(int64_t)mu * n + e] * ra(Q_DRDN + mu, k, e);
    aN[(int64_t)nu * n + e] += g[(int64_t)k * n + e] - yt * diag;
  }
  aP[e] = lk ? y[e] : -yt * (rb(Q_R, 0, e) - d.dRdp[e]) / dt;
}

// Objective increment: sum over listed cells of sum_nu cw_nu dN (one thread,
// fixed order)
__global__ void k_adj_objective(int ncells, const int* __restrict__ cells, const double* __restrict__ objw_cells,
                                const double* __restrict__ cw, int n, int nc, const double* __restrict__ dN,
                                double* __restrict__ J) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double s = 0;
  for (int j = 0; j < ncells; ++j)
    for (int nu = 0; nu < nc; ++nu) s += objw_cells[j] * cw[nu] * dN[(int64_t)nu * n + cells[j]];
  *J += s;
}

}  // namespace

// ----------------------------------------------------------------------
// A 1D tensor map of n elements (boxes of TMA_BOX elements, zero fill past
// the end) for cp.async.bulk.tensor; false when the driver offers no encoder.
static bool tensor_map_1d(CUtensorMap* m, void* base, uint64_t n, CUtensorMapDataType type) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    cudaGetLastError();
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode || n == 0 || n > (1ull << 32)) return false;
  cuuint64_t dim[1] = {n}, stride[1] = {0};
  cuuint32_t box[1] = {(cuuint32_t)TMA_BOX}, es[1] = {1};
  return encode(m, type, 1, base, dim, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct HostFunc {
  DFunc d{};
  DeviceBuffer<double> coord[3], data;
};

static void upload_func(Context& ctx, const rsg_function& f, HostFunc& h) {
  h.d.kind = f.kind;
  h.d.dim = f.dim;
  h.d.value = f.value;
  if (f.kind == RSG_FN_CONSTANT) return;
  if (f.kind != RSG_FN_TABLE && f.kind != RSG_FN_EVEN_TABLE) throw Error(RSG_BAD_ARG, "unknown function kind");
  if (f.dim < 1 || f.dim > 3) throw Error(RSG_BAD_ARG, "table dimension must be 1..3");
  size_t total = 1;
  for (int d = 0; d < f.dim; ++d) {
    if (f.n[d] < 2) throw Error(RSG_BAD_ARG, "table needs two points per axis");
    h.d.n[d] = f.n[d];
    total *= (size_t)f.n[d];
    std::vector<double> c(f.n[d]);
    if (f.kind == RSG_FN_TABLE) {
      for (int j = 0; j < f.n[d]; ++j) c[j] = f.coord[d][j];
      for (int j = 1; j < f.n[d]; ++j)
        if (c[j] <= c[j - 1]) throw Error(RSG_BAD_ARG, "table coordinates must be increasing");
    } else {
      h.d.offset[d] = f.coord[d][0];
      h.d.delta[d] = (f.coord[d][1] - h.d.offset[d]) / (f.n[d] - 1);
      c[0] = h.d.offset[d];
      for (int j = 1; j < f.n[d]; ++j) c[j] = c[j - 1] + h.d.delta[d];
    }
    h.coord[d].resize(c.size());
    RSG_CUDA(cudaMemcpyAsync(h.coord[d].get(), c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, ctx.stream));
    h.d.coord[d] = h.coord[d].get();
  }
  h.data.resize(total);
  RSG_CUDA(cudaMemcpyAsync(h.data.get(), f.data, sizeof(double) * total, cudaMemcpyHostToDevice, ctx.stream));
  h.d.data = h.data.get();
  ctx.sync();
}

static double fmin_out(const rsg_function& f) {
  if (f.kind == RSG_FN_CONSTANT) return f.value;
  size_t total = 1;
  for (int d = 0; d < f.dim; ++d) total *= (size_t)f.n[d];
  return *std::min_element(f.data, f.data + total);
}
static double fmax_out(const rsg_function& f) {
  if (f.kind == RSG_FN_CONSTANT) return f.value;
  size_t total = 1;
  for (int d = 0; d < f.dim; ++d) total *= (size_t)f.n[d];
  return *std::max_element(f.data, f.data + total);
}

// Per-cell terms of Discretisation.residualVolumeFactor and throughputFactor
// (numerics/Discretisation.java:966-998), reduced by maximum: |R| / (V phi)
// with the porosity of calculateRockProperties, and sum_nu |dN_nu| / N_prev
// with dN zero in locked cells.  Both are non-negative (or NaN, which wins as
// Math.max lets it), so their IEEE bit patterns order like their values.
__global__ void k_dt_terms(SimDev d, const int* __restrict__ locked, const double* __restrict__ N_prev,
                           const double* __restrict__ dN, unsigned long long* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const int n = d.n;
  const double c = d.cr[i];
  const double dpp = d.p[i] - d.p0[i];
  const double phi = d.phi0[i] * (1 + c * dpp + c * c * dpp * dpp / 2);
  const double Vp = d.vol[i] * phi;
  const double r = fabs(d.R[i]) / Vp;
  double Ni = 0, dNi = 0;
  for (int nu = 0; nu < d.nc; ++nu) Ni += N_prev[(int64_t)nu * n + i];
  if (!locked[i])
    for (int nu = 0; nu < d.nc; ++nu) dNi += fabs(dN[(int64_t)nu * n + i]);
  const double t = dNi / Ni;
  atomicMax(out, (unsigned long long)__double_as_longlong(r));
  atomicMax(out + 1, (unsigned long long)__double_as_longlong(t));
}

struct Sim {
  Context* ctx;
  Mesh* mesh;
  rsg_runspec spec;
  int n, nc, nconn;
  HostFunc funcs[11];
  int rf_kind = RSG_RF_COREY;
  HostFunc rock_tab[7];  // krw, krg, krow, krog, kro, pcow, pcgo
  // TMA staging of the flux assembly (k_flux_conn_tma): 1D tensor maps of
  // the MD lists and the number of 256-entry boxes a block of connections needs
  CUtensorMap tm_el{}, tm_k{};
  int tma_chunks = 0;
  HostFunc initT, initC[NCM];
  DFluid fl{};
  DCorey co{};
  DeviceBuffer<double> phi0, cr, bf, zc;
  DeviceBuffer<double> p, p0, T, N, phN, phdVdN, S, rho, lambda, Cxi, xi, R, dRdp, dRdN, pcow, pcgo;
  DeviceBuffer<int> present, flag, locked, src_ptr, src_id, bad_row, fixed_id;
  DeviceBuffer<double> src_q, fixed_T, fixed_C;
  DeviceBuffer<double> rho_cs, u, Jh, Jt, rh, rt, cf, dNbuf, part;
  DeviceBuffer<int> up;
  DeviceBuffer<double> p_prev, p0_prev, T_prev, R_prev, N_prev, dp, b;
  DeviceBuffer<double> rawJ, rawB;
  DeviceBuffer<unsigned long long> dpmax_bits;
  DeviceBuffer<double> dp0;
  rsg_csr A;
  SolverPtr solver;
  DeviceBuffer<DCubic> cubic;     // compositional fluid (empty: black-oil)
  HostFunc cubic_w[2];
  double time = 0, last_dt = 0;  // Field.t and the last attempted step
  int last_newton = 0;           // PressureNewtonRaphson.pressureIterations
  DeviceBuffer<unsigned long long> dt_terms;
  std::vector<double> h_src_total;  // dt-independent sum of regular source rates per component
  bool keep_jacobian = false;

  SimDev dev() {
    SimDev d;
    d.n = n;
    d.nc = nc;
    d.nconn = nconn;
    d.fl = fl;
    d.co = co;
    d.rf_kind = rf_kind;
    d.krw = rock_tab[0].d;
    d.krg = rock_tab[1].d;
    d.krow = rock_tab[2].d;
    d.krog = rock_tab[3].d;
    d.kro = rock_tab[4].d;
    d.pcow_t = rock_tab[5].d;
    d.pcgo_t = rock_tab[6].d;
    d.cub = cubic.size() ? cubic.get() : nullptr;
    d.phi0 = phi0.get();
    d.cr = cr.get();
    d.vol = mesh->evol.get();
    d.bf = bf.get();
    d.p = p.get();
    d.p0 = p0.get();
    d.T = T.get();
    d.N = N.get();
    d.phN = phN.get();
    d.phdVdN = phdVdN.get();
    d.S = S.get();
    d.rho = rho.get();
    d.lambda = lambda.get();
    d.Cxi = Cxi.get();
    d.xi = xi.get();
    d.R = R.get();
    d.dRdp = dRdp.get();
    d.dRdN = dRdN.get();
    d.pcow = pcow.get();
    d.pcgo = pcgo.get();
    d.present = present.get();
    d.flag = flag.get();
    return d;
  }
  ConnDev cdev() {
    return ConnDev{mesh->conn.get(), mesh->md_ptr.get(), mesh->md_elem.get(), mesh->md_k.get(),
                   rho_cs.get(),     u.get(),            up.get()};
  }
  AsmDev adev() {
    return AsmDev{mesh->cell_conn.get(), mesh->cell_conn_ptr.get(), mesh->md_ptr.get(), mesh->md_pos_here.get(),
                  mesh->md_pos_there.get(), A.m.rowptr.get(), A.m.diag.get(), src_ptr.get(), src_id.get(),
                  src_q.get(), locked.get(), p_prev.get(), R_prev.get()};
  }

  void check_flag() {
    int h = 0;
    RSG_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (h == FL_DRDP) throw Error(RSG_PHYSICS, "dR/dp must be positive (check PVT data or datum depth/pressure)");
    if (h == FL_NO_WATER) throw Error(RSG_PHYSICS, "Water is not present");
    if (h == FL_TMA) throw Error(RSG_TIMEOUT, "the staging copies of the flux assembly did not complete");
    if (h == FL_CUBIC + 2) throw Error(RSG_SINGULAR, "MatrixSingularException in the flash");
    if (h > FL_CUBIC) throw Error(RSG_PHYSICS, "cubic equation of state failed (code " + std::to_string(h - FL_CUBIC) + ")");
    if (h) throw Error(RSG_PHYSICS, "equation-of-state data check failed (code " + std::to_string(h) + ")");
  }

  void secondaries() {
    SimDev d = dev();
    RSG_LAUNCH(*ctx, "cv", k_cv, blocks_for(n, 128), 128, 0, d);
    RSG_LAUNCH(*ctx, "cs", k_cs, blocks_for(nconn, 128), 128, 0, d, cdev());
  }

  void copy(const DeviceBuffer<double>& a, DeviceBuffer<double>& b, int64_t count) {
    RSG_LAUNCH(*ctx, "copy", k_copy, blocks_for(count, 256), 256, 0, count, a.get(), b.get());
  }

  void store_state() {
    copy(p, p_prev, n);
    copy(p0, p0_prev, n);
    copy(T, T_prev, n);
    copy(R, R_prev, n);
    copy(N, N_prev, (int64_t)nc * n);
  }

  // Discretisation.solve(dt) in phases, so that ensembles can run the
  // pressure solves of many members in one launch: step_begin, then per
  // Newton iteration newton_assemble, a pressure solve of (A, b) into dp,
  // newton_finish (true once converged), and step_end.
  int nt_its = 0, nt_lin = 0;
  double nt_dpMax = 0, nt_dp0 = 0;

  void step_begin(double dt) {
    if (!(dt > 0)) throw Error(RSG_BAD_ARG, "time step must be positive");
    store_state();
    time += dt;  // field.changeTime(dt)
    last_dt = dt;
    nt_its = nt_lin = 0;
    nt_dpMax = nt_dp0 = 0;
  }

  // assemblePressureJacobian + LinearSolver's zeroRows/sign, dp = 0, and
  // the preconditioner's setMatrix
  void newton_assemble(double dt) {
    SimDev d = dev();
    if (tma_chunks > 0)
      RSG_LAUNCH(*ctx, "flux_conn", k_flux_conn_tma, blocks_for(nconn, FLUX_BLOCK), FLUX_BLOCK,
                 (size_t)tma_chunks * TMA_BOX * (sizeof(int) + 3 * sizeof(double)), d, cdev(), Jh.get(), Jt.get(),
                 rh.get(), rt.get(), tm_el, tm_k, tma_chunks);
    else
      RSG_LAUNCH(*ctx, "flux_conn", k_flux_conn, blocks_for(nconn, 128), 128, 0, d, cdev(), Jh.get(), Jt.get(),
                 rh.get(), rt.get());
    RSG_LAUNCH(*ctx, "assemble_rows", k_assemble_rows, blocks_for(n, 128), 128, 0, d, adev(), Jh.get(), Jt.get(),
               rh.get(), rt.get(), dt, A.m.val.get(), b.get(), keep_jacobian ? rawJ.get() : nullptr,
               keep_jacobian ? rawB.get() : nullptr);
    A.m.sell_dirty = true;
    RSG_LAUNCH(*ctx, "zero", k_zero, blocks_for(n, 256), 256, 0, (int64_t)n, dp.get());
    solver_setup(*solver, A.m);
  }

  // updatePressure, calculateSecondaries and the stop test; true once the
  // Newton loop has converged
  bool newton_finish(const rsg_solve_info& si) {
    nt_lin += si.iterations;
    SimDev d = dev();
    RSG_CUDA(cudaMemsetAsync(dpmax_bits.get(), 0, sizeof(unsigned long long), ctx->stream));
    int big = INT32_MAX;
    RSG_CUDA(cudaMemcpyAsync(bad_row.get(), &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    RSG_LAUNCH(*ctx, "update_pressure", k_update_pressure, blocks_for(n, 256), 256, 0, d, dp.get(), locked.get(),
               p_prev.get(), dpmax_bits.get(), bad_row.get(), dp0.get());
    secondaries();
    unsigned long long bits = 0;
    int bad = 0;
    RSG_CUDA(cudaMemcpyAsync(&bits, dpmax_bits.get(), sizeof(bits), cudaMemcpyDeviceToHost, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(&nt_dp0, dp0.get(), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(&bad, bad_row.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    std::memcpy(&nt_dpMax, &bits, sizeof(double));
    if (bad != INT32_MAX)
      throw Error(RSG_NONPOSITIVE_PRESSURE, "Non-positive pressure in element " + std::to_string(bad));
    check_flag();
    ++nt_its;
    const bool ref_rule = spec.newton_stop_rule == 0;
    const bool conv = ref_rule ? (nt_dp0 < spec.pressure_tolerance) : (nt_dpMax < spec.pressure_tolerance);
    if (conv) return true;
    if (nt_its >= spec.max_nonlinear_pressure_iterations)
      throw Error(RSG_NEWTON_NOT_CONVERGED, "Nonlinear pressure solver failed to converge");
    return false;
  }

  // MolarMassExplicit.solve and the final calculateSecondaries
  void step_end(double dt, rsg_step_info* info) {
    SimDev d = dev();
    RSG_LAUNCH(*ctx, "molar_conn", k_molar_conn, blocks_for(nconn, 128), 128, 0, d, cdev(), cf.get());
    int big = INT32_MAX;
    RSG_CUDA(cudaMemcpyAsync(bad_row.get(), &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    RSG_LAUNCH(*ctx, "molar_cells", k_molar_cells, blocks_for(n, 128), 128, 0, d, adev(), cf.get(), dt, N_prev.get(),
               spec.truncate_negative_moles, bad_row.get(), dNbuf.get());
    int bad = 0;
    RSG_CUDA(cudaMemcpyAsync(&bad, bad_row.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (bad != INT32_MAX) throw Error(RSG_NEGATIVE_MOLES, "Negative number of moles in element " + std::to_string(bad));
    secondaries();
    last_newton = nt_its;
    if (info) {
      info->newton_iterations = nt_its;
      info->linear_iterations = nt_lin;
      info->dp_max = nt_dpMax;
      info->dp0 = nt_dp0;
      info->status = RSG_OK;
      info->mass_balance_error = mass_balance(dt);
    }
    check_flag();
  }

  void step(double dt, rsg_step_info* info) {
    step_begin(dt);
    for (;;) {
      newton_assemble(dt);
      rsg_solve_info si{};
      solver_solve(*solver, A.m, b.get(), dp.get(), &si);
      if (newton_finish(si)) break;
    }
    step_end(dt, info);
  }

  double mass_balance(double dt) {
    // |sum_i dN_i - dt * sum(sources)| / sum_i N_i per component, worst one
    const int nb = 256;
    part.resize((size_t)2 * nb);
    std::vector<double> hp(2 * nb);
    double worst = 0;
    for (int nu = 0; nu < nc; ++nu) {
      RSG_LAUNCH(*ctx, "sum_blocks", k_sum_blocks, nb, 256, 0, (int64_t)n, dNbuf.get() + (int64_t)nu * n, part.get());
      RSG_LAUNCH(*ctx, "sum_blocks", k_sum_blocks, nb, 256, 0, (int64_t)n, N_prev.get() + (int64_t)nu * n,
                 part.get() + nb);
      RSG_CUDA(cudaMemcpyAsync(hp.data(), part.get(), sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, ctx->stream));
      ctx->sync();
      double s = 0, tot = 0;
      for (int q = 0; q < nb; ++q) {
        s += hp[q];
        tot += hp[nb + q];
      }
      s -= dt * h_src_total[nu];
      if (tot > 0) worst = std::max(worst, std::fabs(s) / tot);
    }
    return worst;
  }

  // residual-volume and throughput terms (max over cells)
  void dt_terms_max(double* rmax, double* tmax) {
    dt_terms.resize(2);
    RSG_CUDA(cudaMemsetAsync(dt_terms.get(), 0, 2 * sizeof(unsigned long long), ctx->stream));
    RSG_LAUNCH(*ctx, "dt_terms", k_dt_terms, blocks_for(n, 256), 256, 0, dev(), locked.get(), N_prev.get(),
               dNbuf.get(), dt_terms.get());
    unsigned long long h[2];
    RSG_CUDA(cudaMemcpyAsync(h, dt_terms.get(), sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    std::memcpy(rmax, &h[0], sizeof(double));
    std::memcpy(tmax, &h[1], sizeof(double));
  }

  static double dt_factor(double value, double target, const rsg_dt_control& c) {
    // Discretisation.dtFactor (:1000-1002)
    return (1 + c.lambda) * target / (value + c.lambda * target);
  }

  double throughput_factor(const rsg_dt_control& c) {
    double r, t;
    dt_terms_max(&r, &t);
    return dt_factor(t, c.target_throughput, c);
  }

  double calculate_dt(double dt, const rsg_dt_control& c, rsg_dt_factors* f) {
    // Discretisation.calculateDt (:928-964)
    double rmax, tmax;
    dt_terms_max(&rmax, &tmax);
    const double R = dt_factor(rmax, c.target_residual_volume, c);
    const double NR = dt_factor(last_newton, c.target_nonlinear_iterations, c);
    const double T = dt_factor(tmax, c.target_throughput, c);
    const double dt_R = dt * R, dt_NR = dt * NR, dt_T = dt * T;
    double dtNew = std::numeric_limits<double>::max();
    dtNew = std::min(dtNew, dt_R);
    dtNew = std::min(dtNew, dt_NR);
    dtNew = std::min(dtNew, dt_T);
    dtNew = std::min(dtNew, c.dt_max);
    int limit = 0;
    if (c.dt_max == dtNew) limit = 1;
    else if (dt_R == dtNew) limit = 2;
    else if (dt_NR == dtNew) limit = 3;
    else if (dt_T == dtNew) limit = 4;
    dtNew = std::max(dtNew, c.dt_min);
    if (f) {
      f->residual_volume = R;
      f->pressure_iterations = NR;
      f->throughput = T;
      f->limit = limit;
    }
    return dtNew;
  }

  static bool solver_failure(int st) {
    return st == RSG_NOT_CONVERGED_ITERATIONS || st == RSG_NOT_CONVERGED_DIVERGENCE ||
           st == RSG_NOT_CONVERGED_BREAKDOWN || st == RSG_NONPOSITIVE_PRESSURE || st == RSG_NEGATIVE_MOLES ||
           st == RSG_NEWTON_NOT_CONVERGED;
  }

  int step_to(double end_time, const rsg_dt_control& c, double& dt, rsg_step_to_info& in) {
    // TimeStepper.stepTo (numerics/TimeStepper.java:58-102)
    in = rsg_step_to_info{};
    while (time < end_time) {
      if (dt + time > end_time) dt = end_time - time;  // adjustDtForReporting
      for (;;) {
        rsg_step_info si{};
        int st = RSG_OK;
        try {
          step(dt, &si);
        } catch (const Error& e) {
          st = e.status;
          if (!solver_failure(st)) throw;
        }
        in.status = st;
        if (st == RSG_OK) {
          in.steps++;
          in.newton_iterations += si.newton_iterations;
          in.linear_iterations += si.linear_iterations;
          break;
        }
        if (!(dt > c.dt_min)) {
          in.time = time;
          return st;  // the time step cannot be reduced further
        }
        retract();
        in.retries++;
        const double factor = std::min(1. / 2., throughput_factor(c));
        dt = std::min(std::max(dt * factor, c.dt_min), c.dt_max);
      }
      dt = calculate_dt(dt, c, nullptr);
    }
    in.time = time;
    return RSG_OK;
  }

  void retract() {
    time -= last_dt;  // Field.retract(t - dt, ...)
    copy(p_prev, p, n);
    copy(T_prev, T, n);
    copy(N_prev, N, (int64_t)nc * n);
    secondaries();
    ctx->sync();
  }

  // ---------------------------------------------------------- adjoint ----
  struct Snapshot {
    double time = 0;
    DeviceBuffer<double> p, T, N, phN, phdVdN;
    DeviceBuffer<int> present;
  };
  std::vector<Snapshot> ck;        // state at the first step of every block
  Snapshot adj_end;                // state after the forward run
  Snapshot saved;                  // rsg_sim_save_state
  bool has_saved = false;
  std::vector<double> adj_dt;
  int adj_every = 0;
  bool adj_ready = false;
  DeviceBuffer<double> blk_p, blk_N, blk_p1;  // per step of one block: p^n, N^n, p^{n+1}
  int blk_first = -1;                         // step held in slot 0 of the block buffers
  DeviceBuffer<double> adj_objw, adj_cw, adj_objw_cells, adj_J;
  DeviceBuffer<int> adj_cells;
  int adj_ncells = 0;
  DeviceBuffer<int> inv_ptr, inv_q;  // MD entries of every element, ascending

  void snap(Snapshot& s) {
    s.time = time;
    s.p.resize(n);
    s.T.resize(n);
    s.N.resize((size_t)nc * n);
    s.phN.resize((size_t)nc * 3 * n);
    s.phdVdN.resize((size_t)nc * 3 * n);
    s.present.resize(n);
    copy(p, s.p, n);
    copy(T, s.T, n);
    copy(N, s.N, (int64_t)nc * n);
    copy(phN, s.phN, (int64_t)nc * 3 * n);
    copy(phdVdN, s.phdVdN, (int64_t)nc * 3 * n);
    RSG_CUDA(cudaMemcpyAsync(s.present.get(), present.get(), sizeof(int) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  }

  void unsnap(Snapshot& s) {
    time = s.time;
    copy(s.p, p, n);
    copy(s.T, T, n);
    copy(s.N, N, (int64_t)nc * n);
    copy(s.phN, phN, (int64_t)nc * 3 * n);
    copy(s.phdVdN, phdVdN, (int64_t)nc * 3 * n);
    RSG_CUDA(cudaMemcpyAsync(present.get(), s.present.get(), sizeof(int) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    secondaries();
  }

  // one step of the forward run, keeping p^n, N^n and p^{n+1} in slot j
  void record_step(int j, double dt, rsg_step_info* si) {
    RSG_CUDA(cudaMemcpyAsync(blk_p.get() + (int64_t)j * n, p.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice,
                             ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(blk_N.get() + (int64_t)j * nc * n, N.get(), sizeof(double) * nc * n,
                             cudaMemcpyDeviceToDevice, ctx->stream));
    step(dt, si);
    RSG_CUDA(cudaMemcpyAsync(blk_p1.get() + (int64_t)j * n, p.get(), sizeof(double) * n, cudaMemcpyDeviceToDevice,
                             ctx->stream));
  }

  void forward_record(int nsteps, const double* dts, int every, int ncells, const int* cells, const double* cellw,
                      const double* cw, double* J, rsg_adjoint_info* info) {
    if (cubic.size()) throw Error(RSG_UNSUPPORTED, "the adjoint covers black-oil fluids only");
    if (nc > ADJ_NC) throw Error(RSG_UNSUPPORTED, "the adjoint supports at most 3 components");
    if (nsteps <= 0) throw Error(RSG_BAD_ARG, "at least one step is required");
    for (int s = 0; s < nsteps; ++s)
      if (!(dts[s] > 0)) throw Error(RSG_BAD_ARG, "time steps must be positive");
    if (ncells < 0 || (ncells > 0 && (!cells || !cellw)) || !cw) throw Error(RSG_BAD_ARG, "objective");
    std::vector<double> objw(n, 0.0);
    for (int j = 0; j < ncells; ++j) {
      if (cells[j] < 0 || cells[j] >= n) throw Error(RSG_BAD_ARG, "objective cell out of range");
      objw[cells[j]] += cellw[j];
    }
    adj_ready = false;
    adj_every = std::max(1, std::min(every, nsteps));
    adj_dt.assign(dts, dts + nsteps);
    const int nblocks = (nsteps + adj_every - 1) / adj_every;
    ck.resize(nblocks);
    blk_p.resize((size_t)adj_every * n);
    blk_p1.resize((size_t)adj_every * n);
    blk_N.resize((size_t)adj_every * nc * n);
    adj_objw.resize(n);
    adj_cw.resize(nc);
    adj_ncells = ncells;
    adj_cells.resize(std::max(ncells, 1));
    adj_objw_cells.resize(std::max(ncells, 1));
    adj_J.resize(1);
    RSG_CUDA(cudaMemcpyAsync(adj_objw.get(), objw.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(adj_cw.get(), cw, sizeof(double) * nc, cudaMemcpyHostToDevice, ctx->stream));
    if (ncells) {
      RSG_CUDA(cudaMemcpyAsync(adj_cells.get(), cells, sizeof(int) * ncells, cudaMemcpyHostToDevice, ctx->stream));
      RSG_CUDA(cudaMemcpyAsync(adj_objw_cells.get(), cellw, sizeof(double) * ncells, cudaMemcpyHostToDevice,
                               ctx->stream));
    }
    RSG_CUDA(cudaMemsetAsync(adj_J.get(), 0, sizeof(double), ctx->stream));
    rsg_adjoint_info in{};
    for (int s = 0; s < nsteps; ++s) {
      if (s % adj_every == 0) snap(ck[s / adj_every]);
      rsg_step_info si{};
      record_step(s % adj_every, dts[s], &si);
      in.steps++;
      in.newton_iterations += si.newton_iterations;
      in.linear_iterations += si.linear_iterations;
      RSG_LAUNCH(*ctx, "adj_objective", k_adj_objective, 1, 32, 0, adj_ncells, adj_cells.get(), adj_objw_cells.get(),
                 adj_cw.get(), n, nc, dNbuf.get(), adj_J.get());
    }
    blk_first = (nblocks - 1) * adj_every;
    snap(adj_end);
    double hJ = 0;
    RSG_CUDA(cudaMemcpyAsync(&hJ, adj_J.get(), sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    in.objective = hJ;
    if (J) *J = hJ;
    if (info) *info = in;
    adj_ready = true;
  }

  void build_inverse_md() {
    if (inv_ptr.size() == (size_t)n + 1) return;
    const std::vector<int>& ptr = mesh->h_md_ptr;
    const std::vector<int>& el = mesh->h_md_elem;
    std::vector<int> ip(n + 1, 0), iq(std::max<size_t>(el.size(), 1));
    for (size_t m = 0; m < el.size(); ++m) ip[el[m] + 1]++;
    for (int e = 0; e < n; ++e) ip[e + 1] += ip[e];
    std::vector<int> fill(ip.begin(), ip.end() - 1);
    for (int c = 0; c < nconn; ++c)
      for (int m = ptr[c]; m < ptr[c + 1]; ++m) iq[fill[el[m]]++] = m;
    inv_ptr.resize(n + 1);
    inv_q.resize(iq.size());
    RSG_CUDA(cudaMemcpyAsync(inv_ptr.get(), ip.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(inv_q.get(), iq.data(), sizeof(int) * iq.size(), cudaMemcpyHostToDevice, ctx->stream));
    ctx->sync();
  }

  void backward(double rtol, double* grad_host, double* dJdp0, double* dJdN0, rsg_adjoint_info* info) {
    if (!adj_ready) throw Error(RSG_BAD_ARG, "backward needs a recorded forward run");
    build_inverse_md();
    const int K = 1 + nc, nq = adj_nq(nc);
    const int64_t nmd = mesh->nmd;
    DeviceBuffer<double> aP(n), aN((size_t)nc * n), grad(mesh->g.nel), recA((size_t)nq * K * n),
        recB((size_t)nq * K * n), Q((size_t)nc * n), z((size_t)nc * n), cmd((size_t)std::max<int64_t>(nmd, 1) * K),
        mu((size_t)4 * nconn), g((size_t)K * n), w(n), y(n), phi((size_t)4 * n), jh(std::max<int64_t>(nmd, 1)),
        jt(std::max<int64_t>(nmd, 1));
    DeviceBuffer<int> aflag(1);
    RSG_CUDA(cudaMemsetAsync(aP.get(), 0, sizeof(double) * n, ctx->stream));
    RSG_CUDA(cudaMemsetAsync(aN.get(), 0, sizeof(double) * nc * n, ctx->stream));
    RSG_CUDA(cudaMemsetAsync(grad.get(), 0, sizeof(double) * mesh->g.nel, ctx->stream));
    RSG_CUDA(cudaMemsetAsync(aflag.get(), 0, sizeof(int), ctx->stream));
    Csr jac;
    jac.build(ctx, n, A.m.nnz, A.m.h_rowptr.data(), A.m.h_col.data());
    CsrTranspose tr;
    SolverPtr solver_t = make_solver(ctx, spec.linear_solver, spec.preconditioner, rtol, spec.absolute_tolerance,
                                     spec.divergence_tolerance, spec.max_linear_iterations,
                                     spec.gmres_restart > 0 ? spec.gmres_restart : 30);
    if (spec.inner_iterations > 0) solver_set_inner(*solver_t, spec.inner_iterations, spec.inner_tolerance);
    const AdjConn ac{mesh->md_ptr.get(), mesh->md_elem.get(), mesh->md_k.get(), mesh->conn.get(), rho_cs.get(), up.get()};
    const Rec ra{recA.get(), n, K}, rb{recB.get(), n, K};
    const int nsteps = (int)adj_dt.size();
    const int nblocks = (nsteps + adj_every - 1) / adj_every;
    rsg_adjoint_info in{};
    for (int b = nblocks - 1; b >= 0; --b) {
      const int n0 = b * adj_every, n1 = std::min(n0 + adj_every, nsteps);
      if (blk_first != n0) {  // recompute the block from its checkpoint
        unsnap(ck[b]);
        for (int s = n0; s < n1; ++s) {
          rsg_step_info si{};
          record_step(s - n0, adj_dt[s], &si);
          in.recomputed_steps++;
        }
        blk_first = n0;
      }
      for (int s = n1 - 1; s >= n0; --s) {
        const int j = s - n0;
        const double dt = adj_dt[s];
        const double* pn = blk_p.get() + (int64_t)j * n;
        // state (p^{n+1}, N^n) and its secondaries
        copy_ptr(blk_p1.get() + (int64_t)j * n, p.get(), n);
        copy_ptr(blk_N.get() + (int64_t)j * nc * n, N.get(), (int64_t)nc * n);
        secondaries();
        SimDev d = dev();
        AsmDev as = adev();
        RSG_LAUNCH(*ctx, "molar_conn", k_molar_conn, blocks_for(nconn, 128), 128, 0, d, cdev(), cf.get());
        RSG_LAUNCH(*ctx, "adj_inflow", k_adj_inflow, blocks_for(n, 128), 128, 0, d, as, cf.get(), Q.get());
        RSG_LAUNCH(*ctx, "cell_dual", k_cell_dual, blocks_for(n, 128), 128, 0, d, p.get(), N.get(), recA.get());
        RSG_LAUNCH(*ctx, "cell_dual", k_cell_dual, blocks_for(n, 128), 128, 0, d, pn, N.get(), recB.get());
        // moles and objective: weights z^M on Q, their pressure derivatives
        RSG_LAUNCH(*ctx, "adj_z", k_adj_z, blocks_for(n, 256), 256, 0, n, nc, locked.get(), adj_objw.get(),
                   adj_cw.get(), aN.get(), (const double*)nullptr, dRdN.get(), dt, z.get());
        RSG_LAUNCH(*ctx, "adj_conn_vjp", k_adj_conn_vjp, blocks_for(nconn, 128), 128, 0, d, ac, ra, z.get(), cmd.get(),
                   mu.get(), aflag.get());
        RSG_LAUNCH(*ctx, "adj_gather", k_adj_gather, blocks_for(n, 128), 128, 0, n, K, inv_ptr.get(), inv_q.get(),
                   cmd.get(), g.get());
        RSG_LAUNCH(*ctx, "adj_rhs", k_adj_rhs, blocks_for(n, 256), 256, 0, n, aP.get(), g.get(), w.get());
        // exact pressure Jacobian, transposed solve
        RSG_LAUNCH(*ctx, "adj_conn_jac", k_adj_conn_jac, blocks_for(nconn, 128), 128, 0, d, ac, ra, jh.get(), jt.get(),
                   aflag.get());
        RSG_LAUNCH(*ctx, "adj_rows", k_adj_rows, blocks_for(n, 128), 128, 0, d, as, ra, jh.get(), jt.get(), Q.get(),
                   pn, dt, jac.val.get());
        jac.sell_dirty = true;
        tr.update(jac);
        RSG_CUDA(cudaMemsetAsync(y.get(), 0, sizeof(double) * n, ctx->stream));
        rsg_solve_info si{};
        solver_setup(*solver_t, tr.AT);
        solver_solve(*solver_t, tr.AT, w.get(), y.get(), &si);
        in.adjoint_linear_iterations += si.iterations;
        // weights z^M - z^F: moles, objective and pressure equation together
        RSG_LAUNCH(*ctx, "adj_z", k_adj_z, blocks_for(n, 256), 256, 0, n, nc, locked.get(), adj_objw.get(),
                   adj_cw.get(), aN.get(), (const double*)y.get(), dRdN.get(), dt, z.get());
        RSG_LAUNCH(*ctx, "adj_conn_vjp", k_adj_conn_vjp, blocks_for(nconn, 128), 128, 0, d, ac, ra, z.get(), cmd.get(),
                   mu.get(), aflag.get());
        RSG_LAUNCH(*ctx, "adj_gather", k_adj_gather, blocks_for(n, 128), 128, 0, n, K, inv_ptr.get(), inv_q.get(),
                   cmd.get(), g.get());
        RSG_LAUNCH(*ctx, "adj_phi", k_adj_phi, blocks_for(n, 256), 256, 0, d, phi.get());
        mpfa_adjoint(*mesh, 4, mu.get(), phi.get(), 1.0, true, grad.get());
        RSG_LAUNCH(*ctx, "adj_update", k_adj_update, blocks_for(n, 256), 256, 0, d, locked.get(), ra, rb, y.get(),
                   g.get(), Q.get(), pn, dt, aP.get(), aN.get());
        in.backward_steps++;
      }
    }
    int hf = 0;
    RSG_CUDA(cudaMemcpyAsync(&hf, aflag.get(), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    if (hf) throw Error(RSG_UNSUPPORTED, "a connection has more transmissibilities than the adjoint handles");
    check_flag();
    RSG_CUDA(cudaMemcpyAsync(grad_host, grad.get(), sizeof(double) * mesh->g.nel, cudaMemcpyDeviceToHost,
                             ctx->stream));
    if (dJdp0) RSG_CUDA(cudaMemcpyAsync(dJdp0, aP.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (dJdN0)
      RSG_CUDA(cudaMemcpyAsync(dJdN0, aN.get(), sizeof(double) * nc * n, cudaMemcpyDeviceToHost, ctx->stream));
    ctx->sync();
    // leave the simulator at the end of the forward run
    unsnap(adj_end);
    blk_first = -1;
    ctx->sync();
    if (info) *info = in;
  }

  // after a failed backward sweep: the simulator returns to the end of the
  // forward run (the record stays usable); errors here are not reported over
  // the original one
  void abandon_backward() {
    try {
      if (adj_ready) unsnap(adj_end);
      blk_first = -1;
      ctx->sync();
    } catch (...) {
    }
  }

  void copy_ptr(const double* a, double* b, int64_t count) {
    RSG_LAUNCH(*ctx, "copy", k_copy, blocks_for(count, 256), 256, 0, count, a, b);
  }
};

}  // namespace rsg

struct rsg_sim {
  std::unique_ptr<rsg::Sim> s;
};

using rsg::guarded;

extern "C" {

static rsg::DCubic make_dcubic(rsg::Context& c, const rsg_cubic_fluid& f, rsg::HostFunc* w);

static rsg_status sim_create(rsg_ctx* ctx, rsg_mesh* mesh, const rsg_blackoil* fluid, const rsg_cubic_fluid* cubic,
                             const rsg_corey* rf, const double* porosity, const double* compaction, int32_t nsources,
                             const rsg_source* sources, const rsg_initial* init, const rsg_runspec* spec,
                             rsg_sim** out) {
  if (!ctx || !mesh || !fluid || !rf || !porosity || !compaction || !init || !spec || !out) return RSG_BAD_ARG;
  if (nsources < 0 || (nsources > 0 && !sources)) return RSG_BAD_ARG;
  if (!mesh->m.have_md) return RSG_BAD_ARG;
  *out = nullptr;
  rsg_sim* h = new rsg_sim();
  rsg_status st = guarded(&ctx->c, [&] {
    using namespace rsg;
    h->s.reset(new Sim());
    Sim& S = *h->s;
    Context& c = ctx->c;
    S.ctx = &c;
    S.mesh = &mesh->m;
    S.spec = *spec;
    S.n = mesh->m.g.nel;
    S.nconn = mesh->m.g.nconn;
    S.nc = fluid->nc;
    const int n = S.n, nc = S.nc;
    if (nc < 1 || nc > RSG_MAX_COMPONENTS) throw Error(RSG_BAD_ARG, "component count");
    // fluid (BlackOilEquationOfState constructor checks)
    const rsg_function* fs[11] = {&fluid->water_density, &fluid->water_viscosity, &fluid->water_enthalpy,
                                  &fluid->bubble_point,  &fluid->dew_point,       &fluid->oil_density,
                                  &fluid->gas_density,   &fluid->oil_viscosity,   &fluid->gas_viscosity,
                                  &fluid->oil_enthalpy,  &fluid->gas_enthalpy};
    for (int q = 0; q < 11; ++q) upload_func(c, *fs[q], S.funcs[q]);
    if (fmin_out(fluid->water_density) <= 0 || fmin_out(fluid->water_viscosity) <= 0 ||
        fmin_out(fluid->oil_density) <= 0 || fmin_out(fluid->gas_density) <= 0 ||
        fmin_out(fluid->oil_viscosity) <= 0 || fmin_out(fluid->gas_viscosity) <= 0)
      throw Error(RSG_BAD_ARG, "densities and viscosities must be positive");
    if (fmin_out(fluid->bubble_point) < 0 || fmax_out(fluid->bubble_point) > 1 || fmin_out(fluid->dew_point) < 0 ||
        fmax_out(fluid->dew_point) > 1)
      throw Error(RSG_BAD_ARG, "bubble/dew point curves must be in [0,1]");
    DFluid& fl = S.fl;
    fl.nc = nc;
    fl.ngO = fl.ngG = 0;
    for (int i = 0; i < nc; ++i) {
      fl.Mw[i] = fluid->molecular_weight[i];
      if (i == 0 && fluid->group[i] != 0) throw Error(RSG_BAD_ARG, "The water component may not be grouped");
      if (i > 0 && fluid->group[i] == 1) fl.O[fl.ngO++] = i;
      else if (i > 0 && fluid->group[i] == 2) fl.G[fl.ngG++] = i;
      else if (i > 0) throw Error(RSG_BAD_ARG, "component has not been grouped");
    }
    DFunc* dst[11] = {&fl.wden, &fl.wvis, &fl.went, &fl.bub, &fl.dew, &fl.oden,
                      &fl.gden, &fl.ovis, &fl.gvis, &fl.oent, &fl.gent};
    for (int q = 0; q < 11; ++q) *dst[q] = S.funcs[q].d;
    if (cubic) {
      const DCubic dc = make_dcubic(c, *cubic, S.cubic_w);
      S.cubic.resize(1);
      RSG_CUDA(cudaMemcpyAsync(S.cubic.get(), &dc, sizeof(DCubic), cudaMemcpyHostToDevice, c.stream));
      c.sync();
    }
    for (int a = 0; a < 3; ++a) {
      S.co.Sr[a] = rf->Sr[a];
      S.co.n[a] = rf->n[a];
      S.co.ke[a] = rf->ke[a];
    }
    S.co.cw = rf->cw;
    S.co.cow = rf->cow;
    S.co.cg = rf->cg;
    S.co.cog = rf->cog;
    S.co.aw = rf->aw;
    S.co.aow = rf->aow;
    S.co.ag = rf->ag;
    S.co.aog = rf->aog;
    for (int i = 0; i < n; ++i)
      if (porosity[i] < 0 || porosity[i] > 1 || compaction[i] < 0) throw Error(RSG_BAD_ARG, "rock data out of range");
    auto up = [&](DeviceBuffer<double>& dbuf, const double* hsrc, size_t count) {
      dbuf.resize(count);
      RSG_CUDA(cudaMemcpyAsync(dbuf.get(), hsrc, sizeof(double) * count, cudaMemcpyHostToDevice, c.stream));
    };
    up(S.phi0, porosity, n);
    up(S.cr, compaction, n);
    // body force and centre z
    std::vector<double> centers((size_t)3 * n);
    RSG_CUDA(cudaMemcpyAsync(centers.data(), mesh->m.ecenter.get(), sizeof(double) * 3 * n, cudaMemcpyDeviceToHost,
                             c.stream));
    c.sync();
    std::vector<double> bfh(n), zh(n);
    for (int i = 0; i < n; ++i) {
      double x = centers[3 * i], y = centers[3 * i + 1], z = centers[3 * i + 2];
      double distance = (spec->ax - x) * (spec->ax - x) + (spec->ay - y) * (spec->ay - y);
      bfh[i] = G_ACC * z - (spec->omega * spec->omega / 2) * distance;
      zh[i] = z;
    }
    up(S.bf, bfh.data(), n);
    up(S.zc, zh.data(), n);
    // state buffers
    for (auto* b : {&S.p, &S.p0, &S.T, &S.R, &S.dRdp, &S.pcow, &S.pcgo, &S.p_prev, &S.p0_prev, &S.T_prev, &S.R_prev,
                    &S.dp, &S.b})
      b->resize(n);
    S.N.resize((size_t)nc * n);
    S.N_prev.resize((size_t)nc * n);
    S.dRdN.resize((size_t)nc * n);
    S.dNbuf.resize((size_t)nc * n);
    S.phN.resize((size_t)nc * 3 * n);
    S.phdVdN.resize((size_t)nc * 3 * n);
    S.Cxi.resize((size_t)nc * 3 * n);
    for (auto* b : {&S.S, &S.rho, &S.lambda, &S.xi}) b->resize((size_t)3 * n);
    RSG_CUDA(cudaMemsetAsync(S.phN.get(), 0, sizeof(double) * S.phN.size(), c.stream));
    RSG_CUDA(cudaMemsetAsync(S.phdVdN.get(), 0, sizeof(double) * S.phdVdN.size(), c.stream));
    S.present.resize(n);
    RSG_CUDA(cudaMemsetAsync(S.present.get(), 0, sizeof(int) * n, c.stream));
    S.flag.resize(1);
    RSG_CUDA(cudaMemsetAsync(S.flag.get(), 0, sizeof(int), c.stream));
    S.bad_row.resize(1);
    S.dpmax_bits.resize(1);
    S.dp0.resize(1);
    const int64_t nmd = mesh->m.nmd;
    S.rho_cs.resize((size_t)3 * S.nconn);
    S.u.resize((size_t)3 * S.nconn);
    S.up.resize((size_t)3 * S.nconn);
    S.Jh.resize(std::max<int64_t>(nmd, 1));
    S.Jt.resize(std::max<int64_t>(nmd, 1));
    S.rh.resize(S.nconn);
    S.rt.resize(S.nconn);
    S.cf.resize((size_t)nc * S.nconn);
    // TMA staging of the flux assembly: the boxes a block of FLUX_BLOCK
    // connections needs (RSG_FLUX_TMA=0 keeps the plain-load kernel)
    {
      const char* env = getenv("RSG_FLUX_TMA");
      const auto& mp = mesh->m.h_md_ptr;
      int chunks = 0;
      if (!(env && env[0] == '0') && S.nconn > 0 && (int64_t)mp.size() > S.nconn) {
        for (int q0 = 0; q0 < S.nconn; q0 += FLUX_BLOCK) {
          const int m0 = mp[q0], m1 = mp[std::min(q0 + FLUX_BLOCK, S.nconn)];
          chunks = std::max(chunks, (m1 - (m0 & ~1) + TMA_BOX - 1) / TMA_BOX);
          chunks = std::max(chunks, (m1 - (m0 & ~3) + TMA_BOX - 1) / TMA_BOX);
        }
        const size_t smem = (size_t)chunks * TMA_BOX * (sizeof(int) + 3 * sizeof(double));
        const bool ok = smem <= 200 * 1024 &&
                        tensor_map_1d(&S.tm_el, mesh->m.md_elem.get(), (uint64_t)nmd, CU_TENSOR_MAP_DATA_TYPE_INT32) &&
                        tensor_map_1d(&S.tm_k, mesh->m.md_k.get(), (uint64_t)nmd, CU_TENSOR_MAP_DATA_TYPE_FLOAT64) &&
                        cudaFuncSetAttribute(k_flux_conn_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024) == cudaSuccess;
        cudaGetLastError();
        S.tma_chunks = ok ? chunks : 0;
      }
    }
    // sources
    std::vector<std::vector<int>> cell_src(n);
    std::vector<double> q((size_t)std::max(nsources, 1) * RSG_MAX_COMPONENTS, 0.0);
    std::vector<int> lockh(n, 0), fixed(n, -1);
    std::vector<double> fT(std::max(nsources, 1), 0.0), fC((size_t)std::max(nsources, 1) * RSG_MAX_COMPONENTS, 0.0);
    S.h_src_total.assign(nc, 0.0);
    for (int s = 0; s < nsources; ++s) {
      const rsg_source& src = sources[s];
      if (src.num_elements < 0 || (src.num_elements > 0 && !src.elements)) throw Error(RSG_BAD_ARG, "source elements");
      for (int a = 0; a < src.num_elements; ++a)
        if (src.elements[a] < 0 || src.elements[a] >= n) throw Error(RSG_BAD_ARG, "source element out of range");
      if (src.type == RSG_SOURCE_REGULAR) {
        for (int nu = 0; nu < nc; ++nu) {
          if (src.q[nu] < 0) throw Error(RSG_BAD_ARG, "Mass source cannot be negative");
          q[(size_t)s * RSG_MAX_COMPONENTS + nu] = src.q[nu];
          S.h_src_total[nu] += src.q[nu] * src.num_elements;
        }
        for (int a = 0; a < src.num_elements; ++a) cell_src[src.elements[a]].push_back(s);
      } else if (src.type == RSG_SOURCE_FIXED) {
        double C[RSG_MAX_COMPONENTS], sum = 0;
        for (int nu = 0; nu < nc; ++nu) {
          if (src.fraction[nu] < 0) throw Error(RSG_BAD_ARG, "Fraction of component cannot be negative");
          C[nu] = src.fraction[nu];
          sum += C[nu];
        }
        if (sum == 0) {
          C[0] = 1;
          sum = 1;
        }
        for (int nu = 0; nu < nc; ++nu) fC[(size_t)s * RSG_MAX_COMPONENTS + nu] = C[nu] / sum;
        if (src.temperature < 0) throw Error(RSG_BAD_ARG, "Temperature cannot be negative");
        fT[s] = src.temperature;
        for (int a = 0; a < src.num_elements; ++a) {
          lockh[src.elements[a]] = 1;
          fixed[src.elements[a]] = s;
        }
      } else
        throw Error(RSG_UNSUPPORTED, "source type not supported (outlet sources are broken in RS)");
    }
    std::vector<int> sptr(n + 1, 0), sid;
    for (int i = 0; i < n; ++i) {
      sptr[i + 1] = sptr[i] + (int)cell_src[i].size();
      for (int s : cell_src[i]) sid.push_back(s);
    }
    if (sid.empty()) sid.push_back(0);
    S.src_ptr.resize(n + 1);
    S.src_id.resize(sid.size());
    S.locked.resize(n);
    S.fixed_id.resize(n);
    RSG_CUDA(cudaMemcpyAsync(S.src_ptr.get(), sptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(S.src_id.get(), sid.data(), sizeof(int) * sid.size(), cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(S.locked.get(), lockh.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    RSG_CUDA(cudaMemcpyAsync(S.fixed_id.get(), fixed.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c.stream));
    up(S.src_q, q.data(), q.size());
    up(S.fixed_T, fT.data(), fT.size());
    up(S.fixed_C, fC.data(), fC.size());
    // initial values (field/InitialValues.java)
    if (init->datum_pressure <= 0) throw Error(RSG_BAD_ARG, "Datum pressure must be positive");
    upload_func(c, init->temperature, S.initT);
    for (int nu = 0; nu < nc; ++nu) upload_func(c, init->fraction[nu], S.initC[nu]);
    InitDev in{};
    in.datum_depth = init->datum_depth;
    in.datum_pressure = init->datum_pressure;
    in.temperature = S.initT.d;
    for (int nu = 0; nu < nc; ++nu) in.frac[nu] = S.initC[nu].d;
    in.zc = S.zc.get();
    in.fixed_id = S.fixed_id.get();
    in.fixed_T = S.fixed_T.get();
    in.fixed_C = S.fixed_C.get();
    RSG_LAUNCH(c, "init_volume_balance", k_init, blocks_for(n, 64), 64, 0, S.dev(), in);
    S.secondaries();
    S.check_flag();
    // LinearSolver(runSpec, mesh, locked)
    S.A.m.build(&c, n, (int)mesh->m.h_pcol.size(), mesh->m.h_prow.data(), mesh->m.h_pcol.data());
    for (int i = 0; i < n; ++i)
      if (S.A.m.h_diag[i] < 0) throw Error(RSG_MISSING_DIAGONAL, "pressure pattern lacks a diagonal");
    S.solver = make_solver(&c, spec->linear_solver, spec->preconditioner, spec->relative_tolerance,
                                   spec->absolute_tolerance, spec->divergence_tolerance, spec->max_linear_iterations,
                                   spec->gmres_restart > 0 ? spec->gmres_restart : 30);
    if (spec->inner_iterations > 0) solver_set_inner(*S.solver, spec->inner_iterations, spec->inner_tolerance);
    c.sync();
  });
  if (st != RSG_OK) {
    delete h;
    return st;
  }
  *out = h;
  return RSG_OK;
}

rsg_status rsg_sim_create(rsg_ctx* ctx, rsg_mesh* mesh, const rsg_blackoil* fluid, const rsg_corey* rf,
                          const double* porosity, const double* compaction, int32_t nsources,
                          const rsg_source* sources, const rsg_initial* init, const rsg_runspec* spec, rsg_sim** out) {
  return sim_create(ctx, mesh, fluid, nullptr, rf, porosity, compaction, nsources, sources, init, spec, out);
}

rsg_status rsg_sim_create_cubic(rsg_ctx* ctx, rsg_mesh* mesh, const rsg_cubic_fluid* fluid, const rsg_corey* rf,
                                const double* porosity, const double* compaction, int32_t nsources,
                                const rsg_source* sources, const rsg_initial* init, const rsg_runspec* spec,
                                rsg_sim** out) {
  if (!fluid) return RSG_BAD_ARG;
  // the black-oil record carries what the simulator shares between fluids:
  // component count, molecular weights, grouping; its functions are unused
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
  return sim_create(ctx, mesh, &carrier, fluid, rf, porosity, compaction, nsources, sources, init, spec, out);
}

rsg_status rsg_sim_destroy(rsg_sim* s) {
  if (!s) return RSG_BAD_ARG;
  if (s->s) cudaStreamSynchronize(s->s->ctx->stream);
  delete s;
  return RSG_OK;
}

rsg_status rsg_sim_step(rsg_sim* s, double dt, rsg_step_info* info) {
  if (!s) return RSG_BAD_ARG;
  rsg_status st = guarded(s->s->ctx, [&] { s->s->step(dt, info); });
  if (info && st != RSG_OK) info->status = st;
  return st;
}

rsg_status rsg_ensemble_step(int32_t count, rsg_sim* const* sims, const double* dt, int32_t max_concurrent,
                             rsg_step_info* infos, int32_t* statuses) {
  if (count < 0 || (count > 0 && (!sims || !dt))) return RSG_BAD_ARG;
  std::set<rsg::Context*> ctxs;
  for (int i = 0; i < count; ++i) {
    if (!sims[i]) return RSG_BAD_ARG;
    if (!ctxs.insert(sims[i]->s->ctx).second) return RSG_BAD_ARG;  // members must not share a context
  }
  const int workers = std::max(1, max_concurrent > 0 ? std::min<int>(max_concurrent, count) : count);
  std::atomic<int> next{0};
  std::vector<rsg_status> st(count, RSG_OK);
  auto work = [&]() {
    for (;;) {
      const int i = next++;
      if (i >= count) return;
      rsg::Sim& m = *sims[i]->s;
      rsg_step_info inf{};
      st[i] = guarded(m.ctx, [&] {
        RSG_CUDA(cudaSetDevice(m.ctx->device));
        m.step(dt[i], &inf);
      });
      inf.status = st[i];
      if (infos) infos[i] = inf;
      if (statuses) statuses[i] = st[i];
    }
  };
  std::vector<std::thread> pool;
  for (int w = 1; w < workers && w < count; ++w) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  for (int i = 0; i < count; ++i)
    if (st[i] != RSG_OK) return st[i];
  return RSG_OK;
}

rsg_status rsg_ensemble_step_batched(int32_t count, rsg_sim* const* sims, const double* dt, int32_t precision,
                                     rsg_step_info* infos, int32_t* statuses) {
  if (count < 0 || (count > 0 && (!sims || !dt)) || (precision != 0 && precision != 1)) return RSG_BAD_ARG;
  std::set<rsg::Sim*> seen;
  for (int i = 0; i < count; ++i) {
    if (!sims[i]) return RSG_BAD_ARG;
    if (!seen.insert(sims[i]->s.get()).second) return RSG_BAD_ARG;  // a member listed twice
  }
  std::vector<rsg_status> st(count, RSG_OK);
  std::vector<char> live(count, 1), done(count, 0);
  std::vector<rsg_step_info> inf(count);
  for (int i = 0; i < count; ++i) {
    rsg::Sim& m = *sims[i]->s;
    st[i] = guarded(m.ctx, [&] {
      RSG_CUDA(cudaSetDevice(m.ctx->device));
      m.step_begin(dt[i]);
    });
    if (st[i] != RSG_OK) live[i] = 0;
  }
  for (;;) {
    std::vector<int> act;
    for (int i = 0; i < count; ++i)
      if (live[i] && !done[i]) act.push_back(i);
    if (act.empty()) break;
    std::vector<int> go;
    for (int i : act) {
      rsg::Sim& m = *sims[i]->s;
      st[i] = guarded(m.ctx, [&] {
        RSG_CUDA(cudaSetDevice(m.ctx->device));
        m.newton_assemble(dt[i]);
      });
      if (st[i] != RSG_OK) live[i] = 0;
      else go.push_back(i);
    }
    if (go.empty()) continue;
    std::vector<rsg::EnsSystem> sys;
    for (int i : go) {
      rsg::Sim& m = *sims[i]->s;
      sys.push_back(rsg::EnsSystem{m.ctx, &m.A.m, m.solver.get(), m.b.get(), m.dp.get()});
    }
    std::vector<rsg_solve_info> si;
    std::vector<int> ss;
    rsg_status e = guarded(sims[go[0]]->s->ctx, [&] { rsg::ensemble_solve(sys, precision, si, ss); });
    for (size_t k = 0; k < go.size(); ++k) {
      const int i = go[k];
      rsg::Sim& m = *sims[i]->s;
      if (e != RSG_OK) {
        st[i] = e;
        live[i] = 0;
        continue;
      }
      if (ss[k] != RSG_OK) {  // LinearSolver.solve maps the solver's failure to a SolverFailure
        st[i] = (rsg_status)ss[k];
        live[i] = 0;
        continue;
      }
      bool conv = false;
      st[i] = guarded(m.ctx, [&] {
        RSG_CUDA(cudaSetDevice(m.ctx->device));
        conv = m.newton_finish(si[k]);
      });
      if (st[i] != RSG_OK) live[i] = 0;
      else if (conv) done[i] = 1;
    }
  }
  for (int i = 0; i < count; ++i) {
    if (done[i]) {
      rsg::Sim& m = *sims[i]->s;
      st[i] = guarded(m.ctx, [&] {
        RSG_CUDA(cudaSetDevice(m.ctx->device));
        m.step_end(dt[i], &inf[i]);
      });
    }
    inf[i].status = st[i];
    if (infos) infos[i] = inf[i];
    if (statuses) statuses[i] = st[i];
  }
  for (int i = 0; i < count; ++i)
    if (st[i] != RSG_OK) return st[i];
  return RSG_OK;
}

rsg_status rsg_sim_get_time(rsg_sim* s, double* t) {
  if (!s || !t) return RSG_BAD_ARG;
  *t = s->s->time;
  return RSG_OK;
}

rsg_status rsg_sim_calculate_dt(rsg_sim* s, double dt, const rsg_dt_control* c, double* dt_new, rsg_dt_factors* f) {
  if (!s || !c || !dt_new) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { *dt_new = s->s->calculate_dt(dt, *c, f); });
}

rsg_status rsg_sim_throughput_factor(rsg_sim* s, const rsg_dt_control* c, double* factor) {
  if (!s || !c || !factor) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { *factor = s->s->throughput_factor(*c); });
}

rsg_status rsg_sim_step_to(rsg_sim* s, double end_time, const rsg_dt_control* c, double* dt, rsg_step_to_info* info) {
  if (!s || !c || !dt) return RSG_BAD_ARG;
  rsg_step_to_info loc{};
  rsg_step_to_info& in = info ? *info : loc;
  int st = RSG_OK;
  rsg_status g = guarded(s->s->ctx, [&] { st = s->s->step_to(end_time, *c, *dt, in); });
  if (g != RSG_OK) {
    in.status = g;
    return g;
  }
  return (rsg_status)st;
}

rsg_status rsg_sim_forward(rsg_sim* s, int32_t nsteps, const double* dt, int32_t checkpoint_every, int32_t ncells,
                           const int32_t* cells, const double* cell_weights, const double* component_weights,
                           double* objective, rsg_adjoint_info* info) {
  if (!s || !dt || nsteps <= 0 || checkpoint_every <= 0 || !component_weights) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] {
    s->s->forward_record(nsteps, dt, checkpoint_every, ncells, cells, cell_weights, component_weights, objective, info);
  });
}

rsg_status rsg_sim_backward(rsg_sim* s, double rtol, double* dJ_dlogk, double* dJ_dp0, double* dJ_dN0,
                            rsg_adjoint_info* info) {
  if (!s || !dJ_dlogk || !(rtol > 0)) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] {
    try {
      s->s->backward(rtol, dJ_dlogk, dJ_dp0, dJ_dN0, info);
    } catch (...) {
      s->s->abandon_backward();  // back to the end of the forward run, then report
      throw;
    }
  });
}

rsg_status rsg_sim_retract(rsg_sim* s) {
  if (!s) return RSG_BAD_ARG;
  return guarded(s->s->ctx, [&] { s->s->retract(); });
}

rsg_status rsg_sim_save_state(rsg_sim* s) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    m.snap(m.saved);
    m.ctx->sync();
    m.has_saved = true;
  });
}

rsg_status rsg_sim_restore_state(rsg_sim* s) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (!m.has_saved) throw rsg::Error(RSG_BAD_ARG, "no saved state: call rsg_sim_save_state first");
    m.unsnap(m.saved);
    m.ctx->sync();
    m.check_flag();
  });
}

// Restart files.  RS saves the whole Field object at every report time
// (numerics/Main.java:86-105) and a restarted run keeps only its primary
// variables (field/Field.java:207-262, copyPrimary: time, pressure,
// reference pressure, temperature, moles) and recomputes everything else.
// The file holds exactly those, in this layout (little-endian as written):
//   8 bytes  "RSGRST01"
//   int32    n, nc, 1 (layout version), 0
//   float64  time
//   float64  p[n], p0[n] (reference pressure), T[n], N[nc][n] (component major)
namespace {
constexpr char kRestartMagic[8] = {'R', 'S', 'G', 'R', 'S', 'T', '0', '1'};
}

rsg_status rsg_sim_write_restart(rsg_sim* s, const char* path) {
  if (!s || !path) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    const size_t n = (size_t)m.n, nc = (size_t)m.nc;
    std::vector<double> buf((3 + nc) * n);
    RSG_CUDA(cudaMemcpyAsync(buf.data(), m.p.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(buf.data() + n, m.p0.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(buf.data() + 2 * n, m.T.get(), sizeof(double) * n, cudaMemcpyDeviceToHost, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(buf.data() + 3 * n, m.N.get(), sizeof(double) * nc * n, cudaMemcpyDeviceToHost,
                             m.ctx->stream));
    m.ctx->sync();
    FILE* f = std::fopen(path, "wb");
    if (!f) throw rsg::Error(RSG_BAD_ARG, std::string("cannot write ") + path);
    const int32_t hdr[4] = {m.n, m.nc, 1, 0};
    const bool ok = std::fwrite(kRestartMagic, 1, 8, f) == 8 && std::fwrite(hdr, sizeof hdr, 1, f) == 1 &&
                    std::fwrite(&m.time, sizeof(double), 1, f) == 1 &&
                    std::fwrite(buf.data(), sizeof(double), buf.size(), f) == buf.size();
    if (std::fclose(f) != 0 || !ok) throw rsg::Error(RSG_BAD_ARG, std::string("cannot write ") + path);
  });
}

rsg_status rsg_sim_read_restart(rsg_sim* s, const char* path) {
  if (!s || !path) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw rsg::Error(RSG_BAD_ARG, std::string("cannot read ") + path);
    char magic[8];
    int32_t hdr[4];
    double t = 0;
    const size_t n = (size_t)m.n, nc = (size_t)m.nc;
    std::vector<double> buf((3 + nc) * n);
    bool ok = std::fread(magic, 1, 8, f) == 8 && std::fread(hdr, sizeof hdr, 1, f) == 1;
    ok = ok && std::memcmp(magic, kRestartMagic, 8) == 0 && hdr[0] == m.n && hdr[1] == m.nc && hdr[2] == 1;
    ok = ok && std::fread(&t, sizeof(double), 1, f) == 1 && std::fread(buf.data(), sizeof(double), buf.size(), f) ==
                                                                  buf.size();
    std::fclose(f);
    if (!ok) throw rsg::Error(RSG_BAD_ARG, std::string("not a restart file of this simulator: ") + path);
    RSG_CUDA(cudaMemcpyAsync(m.p.get(), buf.data(), sizeof(double) * n, cudaMemcpyHostToDevice, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(m.p0.get(), buf.data() + n, sizeof(double) * n, cudaMemcpyHostToDevice, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(m.T.get(), buf.data() + 2 * n, sizeof(double) * n, cudaMemcpyHostToDevice, m.ctx->stream));
    RSG_CUDA(cudaMemcpyAsync(m.N.get(), buf.data() + 3 * n, sizeof(double) * nc * n, cudaMemcpyHostToDevice,
                             m.ctx->stream));
    // new control volumes: no phase records from earlier evaluations
    RSG_CUDA(cudaMemsetAsync(m.phN.get(), 0, sizeof(double) * m.phN.size(), m.ctx->stream));
    RSG_CUDA(cudaMemsetAsync(m.phdVdN.get(), 0, sizeof(double) * m.phdVdN.size(), m.ctx->stream));
    RSG_CUDA(cudaMemsetAsync(m.present.get(), 0, sizeof(int) * n, m.ctx->stream));
    m.time = t;
    m.secondaries();
    m.ctx->sync();  // buf goes out of scope
    m.check_flag();
  });
}

rsg_status rsg_sim_walk_shapes(rsg_sim* s, int32_t* shapes) {
  if (!s || !shapes) return RSG_BAD_ARG;
  int v[4] = {0, 0, 0, 0};
  if (!rsg::ilu_walk_shape(rsg::solver_view(*s->s->solver).pc, -1, v)) return RSG_UNSUPPORTED;
  for (int q = 0; q < 4; ++q) shapes[q] = v[q];
  return RSG_OK;
}

rsg_status rsg_sim_set_rock_tables(rsg_sim* s, const rsg_rock_tables* t) {
  if (!s || !t) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (t->kind == RSG_RF_COREY) {
      m.rf_kind = RSG_RF_COREY;
    } else {
      if (t->kind != RSG_RF_TABULAR && t->kind != RSG_RF_THREE_PHASE_TABULAR)
        throw rsg::Error(RSG_BAD_ARG, "unknown rock-fluid kind");
      const int dim = t->kind == RSG_RF_TABULAR ? 1 : 2;
      // TabularRockFluid.getRelPermTable: outputs within [0, 1]
      auto check = [&](const rsg_function& f, bool relperm) {
        if (f.kind == RSG_FN_CONSTANT) {
          if (relperm && (f.value < 0 || f.value > 1))
            throw rsg::Error(RSG_BAD_ARG, "relative permeabilities must have values between 0 and 1");
          return;
        }
        if (f.dim != dim) throw rsg::Error(RSG_BAD_ARG, "rock-fluid table of the wrong dimension");
        if (!relperm) return;
        size_t total = 1;
        for (int a = 0; a < f.dim; ++a) total *= (size_t)std::max(f.n[a], 0);
        for (size_t q = 0; q < total; ++q)
          if (f.data[q] < 0 || f.data[q] > 1)
            throw rsg::Error(RSG_BAD_ARG, "relative permeabilities must have values between 0 and 1");
      };
      const bool two = t->kind == RSG_RF_TABULAR;
      check(t->krw, true);
      check(t->krg, true);
      if (two) {
        check(t->krow, true);
        check(t->krog, true);
      } else {
        check(t->kro, true);
      }
      check(t->pcow, false);
      check(t->pcgo, false);
      const rsg_function* f[7] = {&t->krw, &t->krg, &t->krow, &t->krog, &t->kro, &t->pcow, &t->pcgo};
      for (int q = 0; q < 7; ++q) {
        const bool used = two ? q != 4 : (q != 2 && q != 3);
        rsg_function zero{};
        zero.kind = RSG_FN_CONSTANT;
        rsg::upload_func(*m.ctx, used ? *f[q] : zero, m.rock_tab[q]);
      }
      m.rf_kind = t->kind;
    }
    m.secondaries();
    m.check_flag();
  });
}

rsg_status rsg_sim_get_state(rsg_sim* s, double* p, double* N, double* S) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (p) RSG_CUDA(cudaMemcpyAsync(p, m.p.get(), sizeof(double) * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    if (N)
      RSG_CUDA(cudaMemcpyAsync(N, m.N.get(), sizeof(double) * m.nc * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    if (S) RSG_CUDA(cudaMemcpyAsync(S, m.S.get(), sizeof(double) * 3 * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_sim_set_state(rsg_sim* s, const double* p, const double* N) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (p) RSG_CUDA(cudaMemcpyAsync(m.p.get(), p, sizeof(double) * m.n, cudaMemcpyHostToDevice, m.ctx->stream));
    if (N)
      RSG_CUDA(cudaMemcpyAsync(m.N.get(), N, sizeof(double) * m.nc * m.n, cudaMemcpyHostToDevice, m.ctx->stream));
    m.secondaries();
    m.check_flag();
  });
}

rsg_status rsg_sim_get_jacobian(rsg_sim* s, double* values, double* rhs) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (!m.keep_jacobian) {
      m.keep_jacobian = true;
      m.rawJ.resize(std::max(m.A.m.nnz, 1));
      m.rawB.resize(m.n);
      throw rsg::Error(RSG_BAD_ARG, "Jacobian capture enabled; it is available after the next step");
    }
    if (values)
      RSG_CUDA(cudaMemcpyAsync(values, m.rawJ.get(), sizeof(double) * m.A.m.nnz, cudaMemcpyDeviceToHost,
                               m.ctx->stream));
    if (rhs) RSG_CUDA(cudaMemcpyAsync(rhs, m.rawB.get(), sizeof(double) * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

rsg_status rsg_sim_get_residual_volume(rsg_sim* s, double* R, double* dRdp) {
  if (!s) return RSG_BAD_ARG;
  rsg::Sim& m = *s->s;
  return guarded(m.ctx, [&] {
    if (R) RSG_CUDA(cudaMemcpyAsync(R, m.R.get(), sizeof(double) * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    if (dRdp)
      RSG_CUDA(cudaMemcpyAsync(dRdp, m.dRdp.get(), sizeof(double) * m.n, cudaMemcpyDeviceToHost, m.ctx->stream));
    m.ctx->sync();
  });
}

}  // extern "C"

// EOS constants, ComponentParameters() and HydrocarbonViscosity(), on the host
// in the Java operand order; the water functions go to the device
static rsg::DCubic make_dcubic(rsg::Context& c, const rsg_cubic_fluid& f, rsg::HostFunc* w) {
  if (f.nc < 2 || f.nc > RSG_MAX_COMPONENTS)
    throw rsg::Error(RSG_BAD_ARG, "a cubic fluid has 2..RSG_MAX_COMPONENTS components");
  if (f.eos != RSG_EOS_PR && f.eos != RSG_EOS_SRK) throw rsg::Error(RSG_BAD_ARG, "unknown cubic equation of state");
  if (f.flash_tolerance <= 0) throw rsg::Error(RSG_BAD_ARG, "FlashTolerance must be positive");
  rsg::DCubic d{};
  d.nc = f.nc;
  d.eos = f.eos;
  d.maxit = f.flash_max_iterations > 0 ? f.flash_max_iterations : 1000;
  d.criteria = f.flash_criteria;
  d.tol = f.flash_tolerance;
  if (f.eos == RSG_EOS_PR) {
    d.d1 = -(1 + std::sqrt(2.));
    d.d2 = -(1 - std::sqrt(2.));
    d.OmegaA = 0.457235529;
    d.OmegaB = 0.077796074;
  } else {
    d.d1 = -1;
    d.d2 = 0;
    d.OmegaA = 0.42748;
    d.OmegaB = 0.08664;
  }
  for (int i = 0; i < f.nc; ++i) {
    d.Tc[i] = f.Tc[i];
    d.pc[i] = f.pc[i];
    d.omega[i] = f.omega[i];
    d.Mw[i] = f.Mw[i];
    d.Vc[i] = f.Vc[i];
    d.s[i] = f.shift[i];
    for (int j = 0; j < f.nc; ++j) d.dij[i][j] = f.bic[i * RSG_MAX_COMPONENTS + j];
  }
  for (int i = 1; i < f.nc; ++i) {
    const double w = f.omega[i];
    if (f.eos == RSG_EOS_PR)
      d.mi[i] = w > 0.49 ? 0.379642 + 1.48503 * w - 0.164423 * w * w + 0.016666 * w * w * w
                         : 0.37464 + 1.53226 * w - 0.26992 * w * w;
    else
      d.mi[i] = 0.48508 + 1.55171 * w - 0.15613 * w * w;
    d.bi[i] = d.OmegaB * rsg::CUBIC_R * f.Tc[i] / f.pc[i];
    d.sqrtM[i] = std::sqrt(f.Mw[i]);
    d.zeta_inv[i] = d.sqrtM[i] * std::pow(f.pc[i], 2. / 3) / std::pow(f.Tc[i], 1. / 6);
  }
  for (int k = 0; k < 5; ++k) d.lbc[k] = f.lbc[k];
  rsg::upload_func(c, f.water_density, w[0]);
  rsg::upload_func(c, f.water_viscosity, w[1]);
  d.wden = w[0].d;
  d.wvis = w[1].d;
  return d;
}

static rsg_status cubic_phase_state(rsg_ctx* ctx, const rsg_cubic_fluid* fluid, int32_t n, const double* p,
                                    const double* T, const double* N, double* phases, int32_t* iterations,
                                    int32_t* cell_status) {
  if (!ctx || !fluid || n < 0 || (n > 0 && (!p || !T || !N || !phases))) return RSG_BAD_ARG;
  rsg::Context& c = ctx->c;
  return guarded(&c, [&] {
    const rsg_cubic_fluid& f = *fluid;
    if (n >= (1 << 24)) throw rsg::Error(RSG_UNSUPPORTED, "at most 2^24 - 1 cells per call");
    rsg::HostFunc w[2];
    rsg::DCubic d = make_dcubic(c, f, w);
    if (n == 0) return;
    const int nf = 6 + 2 * f.nc;
    rsg::DeviceBuffer<double> dp(n), dT(n), dN((size_t)f.nc * n), dph((size_t)3 * nf * n);
    rsg::DeviceBuffer<int> dit(n), derr(1), dst(cell_status ? n : 0);
    auto up = [&](double* dst, const double* src, size_t cnt) {
      RSG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * cnt, cudaMemcpyHostToDevice, c.stream));
    };
    up(dp.get(), p, n);
    up(dT.get(), T, n);
    up(dN.get(), N, (size_t)f.nc * n);
    up(dph.get(), phases, (size_t)3 * nf * n);
    const int big = INT32_MAX;
    RSG_CUDA(cudaMemcpyAsync(derr.get(), &big, sizeof(int), cudaMemcpyHostToDevice, c.stream));
    RSG_LAUNCH(c, "cubic_phase_state", rsg::k_cubic_phase_state, rsg::blocks_for(n, 128), 128, 0, d, n, dp.get(),
               dT.get(), dN.get(), dph.get(), dit.get(), derr.get(), cell_status ? dst.get() : nullptr);
    if (cell_status)
      RSG_CUDA(cudaMemcpyAsync(cell_status, dst.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
    RSG_CUDA(cudaMemcpyAsync(phases, dph.get(), sizeof(double) * 3 * nf * n, cudaMemcpyDeviceToHost, c.stream));
    if (iterations)
      RSG_CUDA(cudaMemcpyAsync(iterations, dit.get(), sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
    int herr = 0;
    RSG_CUDA(cudaMemcpyAsync(&herr, derr.get(), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    if (herr != INT32_MAX && !cell_status) {
      const int code = herr >> 24, cell = herr & ((1 << 24) - 1);
      static const char* what[] = {"", "Z <= 0", "MatrixSingularException", "Rachford-Rice did not converge",
                                   "flash did not converge", "negative water density derivative"};
      const rsg_status st = code == rsg::CUBIC_SINGULAR ? RSG_SINGULAR : RSG_PHYSICS;
      throw rsg::Error(st, std::string(what[code < 6 ? code : 0]) + " in cell " + std::to_string(cell));
    }
  });
}

rsg_status rsg_cubic_phase_state(rsg_ctx* ctx, const rsg_cubic_fluid* fluid, int32_t n, const double* p,
                                 const double* T, const double* N, double* phases, int32_t* iterations) {
  return cubic_phase_state(ctx, fluid, n, p, T, N, phases, iterations, nullptr);
}

rsg_status rsg_cubic_phase_state_cells(rsg_ctx* ctx, const rsg_cubic_fluid* fluid, int32_t n, const double* p,
                                       const double* T, const double* N, double* phases, int32_t* iterations,
                                       int32_t* cell_status) {
  if (n > 0 && !cell_status) return RSG_BAD_ARG;
  return cubic_phase_state(ctx, fluid, n, p, T, N, phases, iterations, cell_status);
}
