// Oracle (test infrastructure only): black-oil / Corey property chain,
// control-surface fluxes, volume-balance initialisation and the RS pressure
// time step.  See physics.hpp for the reference file list.
#include "physics.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <memory>
#include <set>

namespace orc {

static const double G_ACC = 9.81;  // util/Constants.java:18

// ------------------------------------------------------------ Function ----
Function::Function(const rsg_function& f) {
  kind = f.kind;
  dim = f.dim;
  value = f.value;
  if (kind == RSG_FN_CONSTANT) return;
  if (dim < 1 || dim > 3) throw Failure(ST_BAD_ARG, "table dimension must be 1..3");
  size_t total = 1;
  for (int d = 0; d < dim; ++d) {
    n[d] = f.n[d];
    if (n[d] < 2) throw Failure(ST_BAD_ARG, "table needs two points per axis");
    total *= (size_t)n[d];
    coord[d].resize(n[d]);
    if (kind == RSG_FN_TABLE) {
      for (int j = 0; j < n[d]; ++j) coord[d][j] = f.coord[d][j];
      for (int j = 1; j < n[d]; ++j)
        if (coord[d][j] <= coord[d][j - 1]) throw Failure(ST_BAD_ARG, "table not sorted");
    } else {
      // EvenLookupTable.readTableCoordinates / createCoordinates (:86-162)
      offset[d] = f.coord[d][0];
      delta[d] = (f.coord[d][1] - offset[d]) / (n[d] - 1);
      coord[d][0] = offset[d];
      for (int j = 1; j < n[d]; ++j) coord[d][j] = coord[d][j - 1] + delta[d];
    }
  }
  data.assign(f.data, f.data + total);
}

int Function::getIndex(int d, double x) const {
  if (kind == RSG_FN_EVEN_TABLE) {
    // EvenLookupTable.getIndex (:164-174)
    int index = (int)((x - offset[d]) / delta[d]);
    if (index < 0) index = 0;
    else if (index > n[d] - 2) index = n[d] - 2;
    return index;
  }
  // LookupTable.getIndex (:408-430)
  const std::vector<double>& index = coord[d];
  const int len = n[d];
  if (x <= index[0]) return 0;
  if (x >= index[len - 2]) return len - 2;
  int begin = 0, end = len - 1;
  while (begin <= end) {
    int mid = (end + begin) / 2;
    if (index[mid] < x) begin = mid + 1;
    else end = mid - 1;
  }
  return begin - 1;
}

double Function::getWeight(int d, int index, double x) const {
  // LookupTable.getWeight (:384-393)
  double mn = coord[d][index], mx = coord[d][index + 1];
  if (x <= mn) return 0;
  if (x >= mx) return 1;
  return (x - mn) / (mx - mn);
}

double Function::evaluate(int nd, const double* x) const {
  if (kind == RSG_FN_CONSTANT) return nd < 0 ? value : 0.0;
  // LookupTable.evaluate (:217-357)
  if (nd >= 0 && !(x[nd] >= coord[nd][0] && x[nd] <= coord[nd][n[nd] - 1])) return 0;
  const int nx = n[0], ny = n[1];
  auto d2 = [&](int i, int j) { return data[i + (size_t)j * nx]; };
  auto d3 = [&](int i, int j, int k) { return data[i + (size_t)j * nx + (size_t)k * nx * ny]; };
  if (dim == 1) {
    int xi = getIndex(0, x[0]);
    double xw = getWeight(0, xi, x[0]);
    double phi1, phi2;
    if (nd == -1) {
      phi1 = 1 - xw;
      phi2 = xw;
    } else {
      double delta_ = coord[0][xi + 1] - coord[0][xi];
      phi1 = -1 / delta_;
      phi2 = 1 / delta_;
    }
    return phi1 * data[xi] + phi2 * data[xi + 1];
  }
  if (dim == 2) {
    int xi = getIndex(0, x[0]), yi = getIndex(1, x[1]);
    double xw = getWeight(0, xi, x[0]), yw = getWeight(1, yi, x[1]);
    double phi1, phi2, phi3, phi4, delta_;
    if (nd == -1) {
      phi1 = (1 - xw) * (1 - yw);
      phi2 = xw * (1 - yw);
      phi3 = (1 - xw) * yw;
      phi4 = xw * yw;
    } else if (nd == 0) {
      delta_ = coord[0][xi + 1] - coord[0][xi];
      phi1 = (-1 + yw) / delta_;
      phi2 = (1 - yw) / delta_;
      phi3 = -yw / delta_;
      phi4 = yw / delta_;
    } else {
      delta_ = coord[1][yi + 1] - coord[1][yi];
      phi1 = (-1 + xw) / delta_;
      phi2 = -xw / delta_;
      phi3 = (1 - xw) / delta_;
      phi4 = xw / delta_;
    }
    return phi1 * d2(xi, yi) + phi2 * d2(xi + 1, yi) + phi3 * d2(xi, yi + 1) + phi4 * d2(xi + 1, yi + 1);
  }
  int xi = getIndex(0, x[0]), yi = getIndex(1, x[1]), zi = getIndex(2, x[2]);
  double xw = getWeight(0, xi, x[0]), yw = getWeight(1, yi, x[1]), zw = getWeight(2, zi, x[2]);
  double phi1, phi2, phi3, phi4, phi5, phi6, phi7, phi8, delta_;
  if (nd == -1) {
    phi1 = (1 - xw) * (1 - yw) * (1 - zw);
    phi2 = xw * (1 - yw) * (1 - zw);
    phi3 = (1 - xw) * yw * (1 - zw);
    phi4 = xw * yw * (1 - zw);
    phi5 = (1 - xw) * (1 - yw) * zw;
    phi6 = xw * (1 - yw) * zw;
    phi7 = (1 - xw) * yw * zw;
    phi8 = xw * yw * zw;
  } else if (nd == 0) {
    delta_ = coord[0][xi + 1] - coord[0][xi];
    phi1 = -(1 - yw) * (1 - zw) / delta_;
    phi2 = (1 - yw) * (1 - zw) / delta_;
    phi3 = -yw * (1 - zw) / delta_;
    phi4 = yw * (1 - zw) / delta_;
    phi5 = -(1 - yw) * zw / delta_;
    phi6 = (1 - yw) * zw / delta_;
    phi7 = -yw * zw / delta_;
    phi8 = yw * zw / delta_;
  } else if (nd == 1) {
    delta_ = coord[1][yi + 1] - coord[1][yi];
    phi1 = -(1 - xw) * (1 - zw) / delta_;
    phi2 = -xw * (1 - zw) / delta_;
    phi3 = (1 - xw) * (1 - zw) / delta_;
    phi4 = xw * (1 - zw) / delta_;
    phi5 = -(1 - xw) * zw / delta_;
    phi6 = -xw * zw / delta_;
    phi7 = (1 - xw) * zw / delta_;
    phi8 = xw * zw / delta_;
  } else {
    delta_ = coord[2][zi + 1] - coord[2][zi];
    phi1 = -(1 - xw) * (1 - yw) / delta_;
    phi2 = -xw * (1 - yw) / delta_;
    phi3 = -(1 - xw) * yw / delta_;
    phi4 = -xw * yw / delta_;
    phi5 = (1 - xw) * (1 - yw) / delta_;
    phi6 = xw * (1 - yw) / delta_;
    phi7 = (1 - xw) * yw / delta_;
    phi8 = xw * yw / delta_;
  }
  return phi1 * d3(xi, yi, zi) + phi2 * d3(xi + 1, yi, zi) + phi3 * d3(xi, yi + 1, zi) +
         phi4 * d3(xi + 1, yi + 1, zi) + phi5 * d3(xi, yi, zi + 1) + phi6 * d3(xi + 1, yi, zi + 1) +
         phi7 * d3(xi, yi + 1, zi + 1) + phi8 * d3(xi + 1, yi + 1, zi + 1);
}

double Function::minOutput() const {
  if (kind == RSG_FN_CONSTANT) return value;
  return *std::min_element(data.begin(), data.end());
}
double Function::maxOutput() const {
  if (kind == RSG_FN_CONSTANT) return value;
  return *std::max_element(data.begin(), data.end());
}

// ---------------------------------------------------------------- EOS ----
void EOSData::setNotPresent(int nc) {
  // EquationOfStateData.setPresent(false) (:122-138)
  present = false;
  V = xi = dVdp = dVdT = h = dhdT = mu = 0;
  for (int i = 0; i < nc; ++i) {
    N[i] = 0;
    dVdN[i] = 0;
  }
}

double EOSData::NT(int nc) const {
  double s = 0;
  for (int i = 0; i < nc; ++i) s += N[i];
  return s;
}

static double moleFraction(const double* N, int nc, int nu) {
  // Composition.getMoleFraction (:102-107); the total is the plain sum.
  double NT = 0;
  for (int i = 0; i < nc; ++i) NT += N[i];
  return NT > 0 ? N[nu] / NT : 0;
}

BlackOil::BlackOil(const rsg_blackoil& f)
    : waterDensity(f.water_density),
      waterViscosity(f.water_viscosity),
      waterEnthalpy(f.water_enthalpy),
      bubblePoint(f.bubble_point),
      dewPoint(f.dew_point),
      oilDensity(f.oil_density),
      gasDensity(f.gas_density),
      oilViscosity(f.oil_viscosity),
      gasViscosity(f.gas_viscosity),
      oilEnthalpy(f.oil_enthalpy),
      gasEnthalpy(f.gas_enthalpy) {
  nc = f.nc;
  if (nc < 1 || nc > RSG_MAX_COMPONENTS) throw Failure(ST_BAD_ARG, "component count");
  for (int i = 0; i < nc; ++i) {
    Mw[i] = f.molecular_weight[i];
    if (i == 0 && f.group[i] != 0) throw Failure(ST_BAD_ARG, "The water component may not be grouped");
    if (i > 0 && f.group[i] == 1) O.push_back(i);
    else if (i > 0 && f.group[i] == 2) G.push_back(i);
    else if (i > 0) throw Failure(ST_BAD_ARG, "component has not been grouped");
  }
  // value checks of WaterEquationOfState.java:45-68 and BlackOilEquationOfState.java:86-139
  if (waterDensity.minOutput() <= 0 || waterViscosity.minOutput() <= 0 || oilDensity.minOutput() <= 0 ||
      gasDensity.minOutput() <= 0 || oilViscosity.minOutput() <= 0 || gasViscosity.minOutput() <= 0)
    throw Failure(ST_BAD_ARG, "densities and viscosities must be positive");
  if (bubblePoint.minOutput() < 0 || bubblePoint.maxOutput() > 1 || dewPoint.minOutput() < 0 ||
      dewPoint.maxOutput() > 1)
    throw Failure(ST_BAD_ARG, "bubble/dew point curves must be in [0,1]");
}

void BlackOil::calculatePhaseState(double p, const double* N, double T, EOSData* data) const {
  double pT[2] = {p, T};
  // WaterEquationOfState.calculatePhaseState (:71-129)
  {
    EOSData& water = data[WATER];
    double Nw = N[0];
    if (Nw > 0) {
      water.present = true;
      double xiw = waterDensity.get(pT);
      double Vw = Nw / xiw;
      if (xiw <= 0) throw Failure(ST_PHYSICS, "water molar density cannot be negative");
      water.xi = xiw;
      water.V = Vw;
      water.N[0] = Nw;
      double dxiw_dp = waterDensity.deriv(0, pT);
      double dxiw_dT = waterDensity.deriv(1, pT);
      if (dxiw_dp < 0) throw Failure(ST_PHYSICS, "Water molar density pressure derivative cannot be negative");
      water.dVdp = -(Vw / xiw) * dxiw_dp;
      water.dVdT = -(Vw / xiw) * dxiw_dT;
      water.dVdN[0] = 1 / xiw;
      double hw = waterEnthalpy.get(pT);
      water.h = hw * xiw;
      double dhw_dT = waterEnthalpy.deriv(1, pT);
      water.dhdT = dhw_dT * xiw + hw * dxiw_dT;
      water.mu = waterViscosity.get(pT);
    } else
      water.setNotPresent(nc);
  }
  EOSData& oil = data[OIL];
  EOSData& gas = data[GAS];
  double No = 0, Ng = 0;
  for (int nu : O) No += N[nu];
  for (int nu : G) Ng += N[nu];
  double NHC = No + Ng;
  double NtTotal = 0;
  for (int i = 0; i < nc; ++i) NtTotal += N[i];

  // inverseGroupComposition (:494-506)
  auto inverseGroup = [&](double Nop, double Ngp, EOSData& e) {
    double Co = No / NtTotal, Cg = Ng / NtTotal;
    if (Co > 0)
      for (int nu : O) e.N[nu] = moleFraction(N, nc, nu) * Nop / Co;
    if (Cg > 0)
      for (int nu : G) e.N[nu] = moleFraction(N, nc, nu) * Ngp / Cg;
  };
  // calculateEnthalpy (:511-528)
  auto enthalpy = [&](double C, double dCdT, double xi, double dxidT, double dxidC, const Function& fn, EOSData& e) {
    double x[3] = {p, C, T};
    double hbar = fn.get(x);
    if (hbar * xi < 0) throw Failure(ST_PHYSICS, "enthalpy density cannot be negative");
    e.h = hbar * xi;
    double dhbar_dT = fn.deriv(2, x);
    double dhbar_dC = 0;
    if (dCdT != 0) dhbar_dC = fn.deriv(1, x);
    e.dhdT = (dhbar_dT + dhbar_dC * dCdT) * xi + hbar * (dxidT + dxidC * dCdT);
  };
  auto viscosity = [&](double C, const Function& fn, EOSData& e) {
    double x[3] = {p, C, T};
    e.mu = fn.get(x);
  };

  if (NHC < 1e-300) {
    oil.setNotPresent(nc);
    gas.setNotPresent(nc);
    return;
  }
  double Cb = 0, Cd = 0;
  double Zo = No / NHC, Zg = Ng / NHC;
  if (Zg <= (Cb = bubblePoint.get(pT))) {
    // calculateSinglePhaseOil (:227-277)
    oil.present = true;
    gas.setNotPresent(nc);
    inverseGroup(No, Ng, oil);
    double Cgo = Ng / NHC;
    double x[3] = {p, Cgo, T};
    double xio = oilDensity.get(x);
    double Vo = (No + Ng) / xio;
    if (xio <= 0) throw Failure(ST_PHYSICS, "oil molar density cannot be negative");
    oil.xi = xio;
    oil.V = Vo;
    double dxio_dp = oilDensity.deriv(0, x), dxio_dC = oilDensity.deriv(1, x), dxio_dT = oilDensity.deriv(2, x);
    double dCgo_dNo = -Cgo / NHC;
    double dCgo_dNg = (1 - Cgo) / NHC;
    double Vo_xio = Vo / xio;
    double dVodp = -Vo_xio * dxio_dp;
    double dVodT = -Vo_xio * dxio_dT;
    double dVodNo = (1 / xio) - Vo_xio * dxio_dC * dCgo_dNo;
    double dVodNg = (1 / xio) - Vo_xio * dxio_dC * dCgo_dNg;
    oil.dVdp = dVodp;
    oil.dVdT = dVodT;
    for (int nu : O) oil.dVdN[nu] = dVodNo;
    for (int nu : G) oil.dVdN[nu] = dVodNg;
    enthalpy(1, 0, xio, dxio_dT, dxio_dC, oilEnthalpy, oil);
    viscosity(Cgo, oilViscosity, oil);
  } else if (Zo <= (Cd = dewPoint.get(pT))) {
    // calculateSinglePhaseGas (:282-332)
    oil.setNotPresent(nc);
    gas.present = true;
    inverseGroup(No, Ng, gas);
    double Cog = No / NHC;
    double x[3] = {p, Cog, T};
    double xig = gasDensity.get(x);
    double Vg = (No + Ng) / xig;
    if (xig <= 0) throw Failure(ST_PHYSICS, "gas molar density cannot be negative");
    gas.xi = xig;
    gas.V = Vg;
    double dxig_dp = gasDensity.deriv(0, x), dxig_dC = gasDensity.deriv(1, x), dxig_dT = gasDensity.deriv(2, x);
    double dCgo_dNo = -(1 - Cog) / NHC;
    double dCgo_dNg = -Cog / NHC;
    double Vg_xig = Vg / xig;
    double dVgdp = -Vg_xig * dxig_dp;
    double dVgdT = -Vg_xig * dxig_dT;
    double dVgdNo = (1 / xig) - Vg_xig * dxig_dC * dCgo_dNo;
    double dVgdNg = (1 / xig) - Vg_xig * dxig_dC * dCgo_dNg;
    gas.dVdp = dVgdp;
    gas.dVdT = dVgdT;
    for (int nu : O) gas.dVdN[nu] = dVgdNo;
    for (int nu : G) gas.dVdN[nu] = dVgdNg;
    enthalpy(1, 0, xig, dxig_dT, dxig_dC, gasEnthalpy, gas);
    viscosity(Cog, gasViscosity, gas);
  } else {
    // calculateTwoPhaseOilGas (:337-489) with Cgo = Cb, Cog = Cd
    oil.present = true;
    gas.present = true;
    double Cgo = Cb, Cog = Cd;
    double L = (Cog - Zo) / (Cog - (1 - Cgo));
    double Noo = L * NHC * (1 - Cgo);
    double Ngo = L * NHC * Cgo;
    double Nog = (1 - L) * NHC * Cog;
    double Ngg = (1 - L) * NHC * (1 - Cog);
    inverseGroup(Noo, Ngo, oil);
    inverseGroup(Nog, Ngg, gas);
    double xo[3] = {p, Cgo, T}, xg[3] = {p, Cog, T};
    double xio = oilDensity.get(xo);
    double xig = gasDensity.get(xg);
    double Vo = (Noo + Ngo) / xio;
    double Vg = (Nog + Ngg) / xig;
    oil.xi = xio;
    gas.xi = xig;
    oil.V = Vo;
    gas.V = Vg;
    double dCgo_dp = bubblePoint.deriv(0, pT), dCog_dp = dewPoint.deriv(0, pT);
    double dCgo_dT = bubblePoint.deriv(1, pT), dCog_dT = dewPoint.deriv(1, pT);
    double dLdp = (1 / (Cog - (1 - Cgo))) * ((1 - L) * dCog_dp - L * (dCgo_dp));
    double dLdT = (1 / (Cog - (1 - Cgo))) * ((1 - L) * dCog_dT - L * (dCgo_dT));
    double dLdNo = (1 / (Cog - (1 - Cgo))) * ((Zo - 1) / NHC);
    double dLdNg = (1 / (Cog - (1 - Cgo))) * (Zo / NHC);
    double dxio_dp = oilDensity.deriv(0, xo), dxio_dC = oilDensity.deriv(1, xo), dxio_dT = oilDensity.deriv(2, xo);
    double dxig_dp = gasDensity.deriv(0, xg), dxig_dC = gasDensity.deriv(1, xg), dxig_dT = gasDensity.deriv(2, xg);
    double dVodp = (Vo / L) * dLdp - (Vo / xio) * (dxio_dp + dxio_dC * dCgo_dp);
    double dVgdp = -(Vg / (1 - L)) * dLdp - (Vg / xig) * (dxig_dp + dxig_dC * dCog_dp);
    double dVodT = (Vo / L) * dLdT - (Vo / xio) * (dxio_dT + dxio_dC * dCgo_dT);
    double dVgdT = -(Vg / (1 - L)) * dLdT - (Vg / xig) * (dxig_dT + dxig_dC * dCog_dT);
    double dVodNo = (1 / xio) * (dLdNo * NHC + L);
    double dVodNg = (1 / xio) * (dLdNg * NHC + L);
    double dVgdNo = (1 / xig) * (-dLdNo * NHC + (1 - L));
    double dVgdNg = (1 / xig) * (-dLdNg * NHC + (1 - L));
    oil.dVdp = dVodp;
    oil.dVdT = dVodT;
    gas.dVdp = dVgdp;
    gas.dVdT = dVgdT;
    for (int nu : O) {
      oil.dVdN[nu] = dVodNo;
      gas.dVdN[nu] = dVgdNo;
    }
    for (int nu : G) {
      oil.dVdN[nu] = dVodNg;
      gas.dVdN[nu] = dVgdNg;
    }
    if (Cog - (1 - Cgo) > 0) throw Failure(ST_PHYSICS, "Error detected in the bubble- and dew-point functions");
    if ((1 - L) * dCog_dp - L * dCgo_dp > 0) throw Failure(ST_PHYSICS, "Liquid fraction must increase with pressure");
    if (dVodp + dVgdp > 0) throw Failure(ST_PHYSICS, "Negative hydrocarbon compressibility detected");
    if (dVodNo + dVgdNo <= 0) throw Failure(ST_PHYSICS, "Hydrocarbon volume must increase with oil moles");
    if (dVodNg + dVgdNg <= 0) throw Failure(ST_PHYSICS, "Hydrocarbon volume must increase with gas moles");
    enthalpy(Cgo, dCgo_dT, xio, dxio_dT, dxio_dC, oilEnthalpy, oil);
    enthalpy(Cog, dCog_dT, xig, dxig_dT, dxig_dC, gasEnthalpy, gas);
    viscosity(Cgo, oilViscosity, oil);
    viscosity(Cog, gasViscosity, gas);
  }
}

// -------------------------------------------------------------- Corey ----
// Math.pow as HotSpot evaluates it for an exponent of exactly 2 (x * x);
// other exponents go through the C library pow (within 1 ulp of Java's).
static double jpow(double x, double y) { return y == 2.0 ? x * x : std::pow(x, y); }

double Corey::effectiveSaturation(int phase, double S) const {
  // CoreyRockFluid.effectiveSaturation (:128-141), deliberately unclamped
  double Se = S;
  Se -= c.Sr[phase];
  double denom = 1;
  for (int p = 0; p < 3; ++p) denom -= c.Sr[p];
  Se /= denom;
  return Se;
}
// TabularRockFluid (rock/TabularRockFluid.java:31-57): relative
// permeability tables must have outputs in [0, 1] (getRelPermTable :52-57),
// capillary pressures default to zero
void Corey::setTables(const rsg_rock_tables& t) {
  if (t.kind == RSG_RF_COREY) {
    kind = RSG_RF_COREY;
    return;
  }
  if (t.kind != RSG_RF_TABULAR && t.kind != RSG_RF_THREE_PHASE_TABULAR) throw Failure(ST_BAD_ARG, "rock-fluid kind");
  const int dim = t.kind == RSG_RF_TABULAR ? 1 : 2;
  auto relperm_table = [&](const rsg_function& f) {
    Function k(f);
    if (f.kind != RSG_FN_CONSTANT && f.dim != dim) throw Failure(ST_BAD_ARG, "relative permeability table dimension");
    if (k.minOutput() < 0 || k.maxOutput() > 1)
      throw Failure(ST_BAD_ARG, "relative permeabilities must have values between 0 and 1");
    return k;
  };
  auto pc_table = [&](const rsg_function& f) {
    if (f.kind != RSG_FN_CONSTANT && f.dim != dim) throw Failure(ST_BAD_ARG, "capillary pressure table dimension");
    return Function(f);
  };
  krw = relperm_table(t.krw);
  krg = relperm_table(t.krg);
  if (t.kind == RSG_RF_TABULAR) {
    krow = relperm_table(t.krow);
    krog = relperm_table(t.krog);
  } else {
    kro = relperm_table(t.kro);
  }
  pcowF = pc_table(t.pcow);
  pcgoF = pc_table(t.pcgo);
  kind = t.kind;
}

void Corey::relperm(const double* S, double* kr) const {
  if (kind == RSG_RF_TABULAR) {
    // TabularRockFluid.calculateRelativePermeability (:60-73)
    kr[WATER] = krw.get(&S[WATER]);
    kr[GAS] = krg.get(&S[GAS]);
    if (S[WATER] <= 0) throw Failure(ST_PHYSICS, "Water is not present");
    const double sow = S[OIL] + S[WATER];
    kr[OIL] = (S[GAS] * krog.get(&sow) + S[WATER] * krow.get(&S[OIL])) / (S[GAS] + S[WATER]);
    return;
  }
  if (kind == RSG_RF_THREE_PHASE_TABULAR) {
    // ThreePhaseTabularRockFluid.calculateRelativePermeability (:72-78)
    const double wg[2] = {S[WATER], S[GAS]};
    kr[WATER] = krw.get(wg);
    kr[GAS] = krg.get(wg);
    kr[OIL] = kro.get(wg);
    return;
  }
  for (int ph = 0; ph < 3; ++ph) kr[ph] = c.ke[ph] * jpow(effectiveSaturation(ph, S[ph]), c.n[ph]);
}
double Corey::pcow(const double* S) const {
  if (kind == RSG_RF_TABULAR) return pcowF.get(&S[WATER]);
  if (kind == RSG_RF_THREE_PHASE_TABULAR) {
    const double wg[2] = {S[WATER], S[GAS]};
    return pcowF.get(wg);
  }
  double Sw = effectiveSaturation(WATER, S[WATER]), So = effectiveSaturation(OIL, S[OIL]);
  double pc = 0;
  if (Sw > 0) pc += c.cw / jpow(Sw, c.aw);
  if (So > 0) pc -= c.cow / jpow(So, c.aow);
  return pc;
}
double Corey::pcgo(const double* S) const {
  if (kind == RSG_RF_TABULAR) return pcgoF.get(&S[GAS]);
  if (kind == RSG_RF_THREE_PHASE_TABULAR) {
    const double wg[2] = {S[WATER], S[GAS]};
    return pcgoF.get(wg);
  }
  double Sg = effectiveSaturation(GAS, S[GAS]), So = effectiveSaturation(OIL, S[OIL]);
  double pc = 0;
  if (Sg > 0) pc += c.cg / jpow(Sg, c.ag);
  if (So > 0) pc -= c.cog / jpow(So, c.aog);
  return pc;
}

// ---------------------------------------------------------- Simulator ----
Simulator::Simulator(const Mesh& m, const rsg_blackoil& fluid, const rsg_corey& rf, const double* poro,
                     const double* comp, int nsources, const rsg_source* src, const rsg_initial& init,
                     const rsg_runspec& sp, const rsg_cubic_fluid* cubicFluid)
    : mesh(&m), eos(fluid), spec(sp) {
  if (cubicFluid) {
    useCubic = true;
    cubic = *cubicFluid;
    cubicWden = Function(cubic.water_density);
    cubicWvis = Function(cubic.water_viscosity);
  }
  rockFluid.c = rf;
  nc = eos.nc;
  const int n = m.numElements();
  phi0.assign(poro, poro + n);
  cr.assign(comp, comp + n);
  heatCap.assign(n, 0.0);
  for (int i = 0; i < n; ++i)
    if (phi0[i] < 0 || phi0[i] > 1 || cr[i] < 0) throw Failure(ST_BAD_ARG, "rock data out of range");
  cv.assign(n, CVState());
  cs.assign(m.numConnections(), CSState());
  omega = sp.omega;
  ax = sp.ax;
  ay = sp.ay;
  std::set<int> lockSet;
  for (int s = 0; s < nsources; ++s) {
    sources.push_back(src[s]);
    sourceElements.emplace_back(src[s].elements, src[s].elements + src[s].num_elements);
    for (int e : sourceElements.back())
      if (e < 0 || e >= n) throw Failure(ST_BAD_ARG, "source element out of range");
    if (src[s].type == RSG_SOURCE_FIXED)
      for (int e : sourceElements.back()) lockSet.insert(e);
  }
  locked.assign(lockSet.begin(), lockSet.end());
  // Field(config, mesh): volume balance in regular, then fixed-source blocks
  volumeBalanceInit(init);
  calculateSecondaries();
  // LinearSolver(runSpec, mesh, locked)
  A = pressure_pattern(m);
  b.assign(n, 0.0);
  x.assign(n, 0.0);
  switch (spec.preconditioner) {
    case RSG_PC_NONE: M.reset(new IdentityPreconditioner()); break;
    case RSG_PC_DIAGONAL: M.reset(new DiagonalPreconditioner()); break;
    case RSG_PC_ILU: M.reset(new ILU()); break;
    case RSG_PC_SSOR: M.reset(new SSOR()); break;
    case RSG_PC_AMG: M.reset(new AMG()); break;
    default: throw Failure(ST_UNSUPPORTED, "preconditioner not available in the oracle");
  }
  p_prev.assign(n, 0);
  T_prev.assign(n, 0);
  R_prev.assign(n, 0);
  N_prev.assign((size_t)nc * n, 0);
  dp.assign(n, 0);
  dN.assign((size_t)nc * n, 0);
}

double Simulator::bodyForce(int el) const {
  // CS.bodyForce (field/CS.java:161-170)
  const Vec3& c = mesh->ecenter[el];
  double distance = (ax - c.x) * (ax - c.x) + (ay - c.y) * (ay - c.y);
  return G_ACC * c.z - (omega * omega / 2) * distance;
}

void Simulator::cvSecondaries(int i) {
  // CV.calculateSecondaries (field/CV.java:375-398)
  CVState& s = cv[i];
  const double V = mesh->evolume[i];
  // calculateFluidProperties (:403-441)
  if (useCubic) cubic_phase_state(cubic, cubicWden, cubicWvis, s.p, s.T, s.N, s.eos);
  else eos.calculatePhaseState(s.p, s.N, s.T, s.eos);
  s.delta = V * heatCap[i];
  for (int ph = 0; ph < 3; ++ph) {
    const EOSData& e = s.eos[ph];
    if (!e.present) {
      s.rho[ph] = 0;
      continue;
    }
    s.delta += e.V * e.dhdT;
    double kg = 0;
    for (int nu = 0; nu < nc; ++nu) kg += eos.Mw[nu] * e.N[nu];
    s.rho[ph] = kg / e.V;
  }
  // calculateRockProperties (:446-459)
  double c = cr[i];
  double dpp = s.p - s.p0;
  s.phi = phi0[i] * (1 + c * dpp + c * c * dpp * dpp / 2);
  double Vf = 0;
  for (int ph = 0; ph < 3; ++ph) Vf += s.eos[ph].V;
  for (int ph = 0; ph < 3; ++ph) s.S[ph] = s.eos[ph].V / Vf;
  // calculateRockFluidProperties (:465-470)
  rockFluid.relperm(s.S, s.kr);
  s.pcow = rockFluid.pcow(s.S);
  s.pcgo = rockFluid.pcgo(s.S);
  // calculateResidualVolume (:475-501)
  double Vp = s.phi * V;
  s.R = Vp;
  s.dRdp = c * Vp;
  s.dRdT = 0;
  for (int nu = 0; nu < nc; ++nu) s.dRdN[nu] = 0;
  for (int ph = 0; ph < 3; ++ph) {
    const EOSData& e = s.eos[ph];
    s.R -= e.V;
    s.dRdp -= e.dVdp;
    s.dRdT -= e.dVdT;
    for (int nu = 0; nu < nc; ++nu) s.dRdN[nu] -= e.dVdN[nu];
  }
  if (s.dRdp <= 0) throw Failure(ST_PHYSICS, "dR/dp must be positive in element " + std::to_string(i + 1));
  // calculatePhaseMobility (:506-516)
  for (int ph = 0; ph < 3; ++ph) {
    s.lambda[ph] = 0;
    double mul = s.eos[ph].mu;
    if (mul != 0) s.lambda[ph] = s.kr[ph] / mul;
  }
  // calculateComponentMobility (:521-536)
  for (int ph = 0; ph < 3; ++ph) {
    const EOSData& e = s.eos[ph];
    for (int nu = 0; nu < nc; ++nu) s.compMob[nu][ph] = moleFraction(e.N, nc, nu) * e.xi * s.lambda[ph];
  }
}

void Simulator::csSecondaries(int c) {
  // CS.calculateSecondaries (field/CS.java:94-155)
  CSState& s = cs[c];
  const CVState& h = cv[mesh->connHere[c]];
  const CVState& t = cv[mesh->connThere[c]];
  for (int ph = 0; ph < 3; ++ph) {
    s.rho[ph] = 0;
    double Sh = h.S[ph], St = t.S[ph];
    double S = Sh + St;
    double av = (Sh * h.rho[ph] + St * t.rho[ph]) / S;
    if (!std::isnan(av)) s.rho[ph] = av;
  }
  for (int ph = 0; ph < 3; ++ph) {
    double D = 0;
    for (auto& tk : mesh->MD[c]) {
      double psi = cv[tk.element].phasePressure(ph) + s.rho[ph] * bodyForce(tk.element);
      D += tk.k * psi;
    }
    int up = (D > 0) ? mesh->connHere[c] : mesh->connThere[c];
    s.upstream[ph] = up;
    s.u[ph] = cv[up].lambda[ph] * D;
  }
}

void Simulator::calculateSecondaries() {
  for (int i = 0; i < mesh->numElements(); ++i) cvSecondaries(i);
  for (int c = 0; c < mesh->numConnections(); ++c) csSecondaries(c);
}

void Simulator::volumeBalance(const rsg_initial& init, const double* C, int i) {
  // Field.volumeBalance (field/Field.java:390-447)
  const int minIters = 3, maxIters = 50;
  double dz = mesh->ecenter[i].z - init.datum_depth;
  cvSecondaries(i);
  CVState& s = cv[i];
  int iters = 0;
  do {
    double dRdNt = 0;
    for (int nu = 0; nu < nc; ++nu) dRdNt += s.dRdN[nu] * C[nu];
    if (dRdNt == 0) throw Failure(ST_PHYSICS, "dR/dN is zero in element " + std::to_string(i + 1));
    double Nt = 0;
    for (int nu = 0; nu < nc; ++nu) Nt += s.N[nu];
    double dNt = -s.R / dRdNt;
    double alpha = 1;
    while (Nt + alpha * dNt < 0) alpha /= 2;
    Nt += alpha * dNt;
    for (int nu = 0; nu < nc; ++nu) s.N[nu] = Nt * C[nu];
    double p = init.datum_pressure;
    for (int ph = 0; ph < 3; ++ph) p -= G_ACC * s.rho[ph] * s.S[ph] * dz;
    s.p = p;
    s.p0 = p;
    cvSecondaries(i);
    iters++;
  } while (iters < minIters || (std::fabs(s.R) > 1.0e-9 && iters < maxIters));
}

void Simulator::volumeBalanceInit(const rsg_initial& init) {
  Function Tz(init.temperature);
  std::vector<Function> Cz;
  for (int nu = 0; nu < nc; ++nu) Cz.emplace_back(init.fraction[nu]);
  if (init.datum_pressure <= 0) throw Failure(ST_BAD_ARG, "Datum pressure must be positive");
  const int n = mesh->numElements();
  for (int i = 0; i < n; ++i) {
    // Field.setInitialState (:307-343)
    double z = mesh->ecenter[i].z;
    CVState& s = cv[i];
    s.p = init.datum_pressure;
    s.p0 = init.datum_pressure;
    s.T = Tz.get(&z);
    double C[RSG_MAX_COMPONENTS];
    double sum = 0;
    for (int nu = 0; nu < nc; ++nu) {
      C[nu] = Cz[nu].get(&z);
      sum += C[nu];
    }
    if (sum == 0) {
      C[0] = 1;
      sum = 1;
    }
    for (int nu = 0; nu < nc; ++nu) {
      C[nu] /= sum;
      s.N[nu] = 1 * C[nu];
    }
    volumeBalance(init, C, i);
  }
  for (size_t q = 0; q < sources.size(); ++q) {
    if (sources[q].type != RSG_SOURCE_FIXED) continue;
    // FixedSource (field/Source.java:65-110): fractions normalised, default water
    double C[RSG_MAX_COMPONENTS];
    double sum = 0;
    for (int nu = 0; nu < nc; ++nu) {
      C[nu] = sources[q].fraction[nu];
      sum += C[nu];
    }
    if (sum == 0) {
      C[0] = 1;
      sum = 1;
    }
    for (int nu = 0; nu < nc; ++nu) C[nu] /= sum;
    for (int i : sourceElements[q]) {
      CVState& s = cv[i];
      s.p = init.datum_pressure;
      s.p0 = init.datum_pressure;
      s.T = sources[q].temperature;
      for (int nu = 0; nu < nc; ++nu) s.N[nu] = 1 * C[nu];
      volumeBalance(init, C, i);
    }
  }
}

void Simulator::storeCurrentState() {
  // Discretisation.storeCurrentState (:231-243)
  const int n = mesh->numElements();
  for (int i = 0; i < n; ++i) {
    p_prev[i] = cv[i].p;
    T_prev[i] = cv[i].T;
    R_prev[i] = cv[i].R;
    for (int nu = 0; nu < nc; ++nu) N_prev[(size_t)nu * n + i] = cv[i].N[nu];
  }
}

void Simulator::assembleFlux() {
  // PressureNewtonRaphson.assemblePressureJacobianFlux (Discretisation.java:459-561), isothermal
  for (int c = 0; c < mesh->numConnections(); ++c) {
    int i = mesh->connHere[c], j = mesh->connThere[c];
    const CVState& h = cv[i];
    const CVState& t = cv[j];
    const CSState& s = cs[c];
    double ri = 0, rj = 0;
    for (auto& tr : mesh->MD[c]) {
      int ik = tr.element;
      double tk = tr.k;
      double bf = bodyForce(ik);
      const CVState& ck = cv[ik];
      double Ji = 0, Jj = 0;
      for (int ph = 0; ph < 3; ++ph) {
        const CVState& up = cv[s.upstream[ph]];
        if (!up.eos[ph].present) continue;
        double psi = ck.phasePressure(ph) + s.rho[ph] * bf;
        for (int nu = 0; nu < nc; ++nu) {
          double phaseCompMob = up.compMob[nu][ph];
          double dRdNhere = h.dRdN[nu];
          double dRdNthere = t.dRdN[nu];
          double dNdt = -phaseCompMob * tk * psi;
          double d2Ndtp = -phaseCompMob * tk;
          ri += dRdNhere * dNdt;
          rj += -dRdNthere * dNdt;
          Ji += dRdNhere * d2Ndtp;
          Jj += -dRdNthere * d2Ndtp;
        }
      }
      A.add(i, ik, Ji);
      A.add(j, ik, Jj);
    }
    b[i] += ri;
    b[j] += rj;
  }
}

void Simulator::assembleDiagonal(double dt) {
  // assemblePressureJacobianDiagonal (:365-401) + assemblePressureRegularSource (:406-424)
  const int n = mesh->numElements();
  for (int i = 0; i < n; ++i) {
    double dpp = cv[i].p - p_prev[i];
    double dRdp = cv[i].dRdp;
    b[i] += (R_prev[i] + dRdp * dpp) / dt;
    A.add(i, i, dRdp / dt);
  }
  for (size_t q = 0; q < sources.size(); ++q) {
    if (sources[q].type != RSG_SOURCE_REGULAR) continue;
    for (int e : sourceElements[q])
      for (int nu = 0; nu < nc; ++nu) b[e] += cv[e].dRdN[nu] * sources[q].q[nu];
  }
}

int Simulator::linearSolve() {
  // LinearSolver.solve (numerics/LinearSolver.java:244-294)
  std::fill(x.begin(), x.end(), 0.0);
  vscale(b, -1);
  lastJ = A.data;
  lastRhs = b;
  zeroRows(A, 1, locked);
  for (int l : locked) b[l] = 0;
  IterationMonitor it;
  it.maxIter = spec.max_linear_iterations;
  it.rtol = spec.relative_tolerance;
  it.atol = spec.absolute_tolerance;
  it.dtol = spec.divergence_tolerance;
  int iters = 0;
  try {
    M->setMatrix(A);
    switch (spec.linear_solver) {
      case RSG_CG: cg_solve(A, b, x, *M, it); break;
      case RSG_BICGSTAB: bicgstab_solve(A, b, x, *M, it); break;
      case RSG_GMRES: gmres_solve(A, b, x, *M, it, spec.gmres_restart > 0 ? spec.gmres_restart : 30); break;
      default: throw Failure(ST_UNSUPPORTED, "linear solver not available in the oracle");
    }
    iters = it.iter;
  } catch (...) {
    A.zero();
    std::fill(b.begin(), b.end(), 0.0);
    throw;
  }
  A.zero();
  std::fill(b.begin(), b.end(), 0.0);
  for (int l : locked) x[l] = 0;
  return iters;
}

double Simulator::updatePressure() {
  // PressureNewtonRaphson.updatePressure (:340-359)
  double dpMax = 0;
  for (int i = 0; i < mesh->numElements(); ++i) {
    double p_old = cv[i].p;
    double p_new = p_old + dp[i];
    if (p_new <= 0) throw Failure(ST_NONPOSITIVE_PRESSURE, "Non-positive pressure in element " + std::to_string(i + 1));
    cv[i].p = p_new;
    dpMax = std::max(dpMax, std::fabs(dp[i] / p_prev[i]));
  }
  return dpMax;
}

void Simulator::molarMass(double dt) {
  // MolarMassExplicit.solve (:769-919)
  const int n = mesh->numElements();
  std::fill(dN.begin(), dN.end(), 0.0);
  double compFlux[RSG_MAX_COMPONENTS];
  for (int c = 0; c < mesh->numConnections(); ++c) {
    int i = mesh->connHere[c], j = mesh->connThere[c];
    for (int nu = 0; nu < nc; ++nu) compFlux[nu] = 0;
    for (int ph = 0; ph < 3; ++ph) {
      const CVState& up = cv[cs[c].upstream[ph]];
      if (!up.eos[ph].present) continue;
      double D = cs[c].u[ph];
      double xi = up.eos[ph].xi;
      for (int nu = 0; nu < nc; ++nu) compFlux[nu] += moleFraction(up.eos[ph].N, nc, nu) * xi * D;
    }
    for (int nu = 0; nu < nc; ++nu) {
      dN[(size_t)nu * n + i] -= dt * compFlux[nu];
      dN[(size_t)nu * n + j] += dt * compFlux[nu];
    }
  }
  for (size_t q = 0; q < sources.size(); ++q) {
    if (sources[q].type != RSG_SOURCE_REGULAR) continue;
    for (int e : sourceElements[q])
      for (int nu = 0; nu < nc; ++nu) dN[(size_t)nu * n + e] += dt * sources[q].q[nu];
  }
  // Per-step mass balance of the explicit update before the locks apply:
  // |sum_i dN_i - dt * sum(sources)| / sum_i N_i, worst component.
  massBalance = 0;
  for (int nu = 0; nu < nc; ++nu) {
    double s = 0, tot = 0;
    for (int i = 0; i < n; ++i) {
      s += dN[(size_t)nu * n + i];
      tot += N_prev[(size_t)nu * n + i];
    }
    for (size_t q = 0; q < sources.size(); ++q)
      if (sources[q].type == RSG_SOURCE_REGULAR) s -= dt * sources[q].q[nu] * (double)sourceElements[q].size();
    if (tot > 0) massBalance = std::max(massBalance, std::fabs(s) / tot);
  }
  dNfull = dN;  // before the locks: moles flowing into locked (Fixed) cells
  for (int l : locked)
    for (int nu = 0; nu < nc; ++nu) dN[(size_t)nu * n + l] = 0;
  for (int i = 0; i < n; ++i)
    for (int nu = 0; nu < nc; ++nu) {
      double Nold = N_prev[(size_t)nu * n + i];
      double Nnew = Nold + dN[(size_t)nu * n + i];
      if (Nnew < 0) {
        if (spec.truncate_negative_moles) Nnew = 0;
        else throw Failure(ST_NEGATIVE_MOLES, "Negative number of moles in element " + std::to_string(i + 1));
      }
      cv[i].N[nu] = Nnew;
    }
}

int Simulator::step(double dt, rsg_step_info* info) {
  // Discretisation.solve (:208-225) with PressureNewtonRaphson.solve (:280-332)
  storeCurrentState();
  time += dt;  // field.changeTime(dt)
  lastDt = dt;
  pressureIterations = 0;
  double dpMax = 0, dpMax_prev = 0, diff = 0;
  int linIts = 0;
  const bool refRule = spec.newton_stop_rule == 0;
  while (true) {
    assembleFlux();
    assembleDiagonal(dt);
    linIts += linearSolve();
    dp = x;
    dpMax_prev = dpMax;
    dpMax = updatePressure();
    calculateSecondaries();
    diff = std::fabs(dpMax_prev - dpMax);
    ++pressureIterations;
    (void)diff;
    bool conv = refRule ? (dp[0] < spec.pressure_tolerance) : (dpMax < spec.pressure_tolerance);
    if (conv) break;
    if (pressureIterations >= spec.max_nonlinear_pressure_iterations)
      throw Failure(ST_NEWTON_NOT_CONVERGED, "Nonlinear pressure solver failed to converge");
  }
  molarMass(dt);
  calculateSecondaries();
  lastLinearIterations = linIts;
  if (info) {
    info->newton_iterations = pressureIterations;
    info->linear_iterations = linIts;
    info->dp_max = dpMax;
    info->dp0 = dp[0];
    info->status = 0;
    double worst = massBalance;
    info->mass_balance_error = worst;
  }
  return pressureIterations;
}

void Simulator::retract() {
  // Discretisation.retractField(dt) -> Field.retract(t - dt, ...) (field/Field.java:535-545)
  time -= lastDt;
  const int n = mesh->numElements();
  for (int i = 0; i < n; ++i) {
    cv[i].p = p_prev[i];
    cv[i].T = T_prev[i];
    for (int nu = 0; nu < nc; ++nu) cv[i].N[nu] = N_prev[(size_t)nu * n + i];
  }
  calculateSecondaries();
}

// Math.max with Java's NaN rule
static double jmax(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  return a >= b ? a : b;
}

double Simulator::dtFactor(double value, double target, const rsg_dt_control& c) const {
  // Discretisation.dtFactor (:1000-1002)
  return (1 + c.lambda) * target / (value + c.lambda * target);
}

double Simulator::residualVolumeFactor(const rsg_dt_control& c) const {
  // :966-978
  double maxR = 0;
  for (int i = 0; i < mesh->numElements(); ++i) {
    double R = cv[i].R;
    double Vp = mesh->evolume[i] * cv[i].phi;
    maxR = jmax(maxR, std::fabs(R) / Vp);
  }
  return dtFactor(maxR, c.target_residual_volume, c);
}

double Simulator::throughputFactor(const rsg_dt_control& c) const {
  // :986-998; N[i] is the state stored at the start of the step
  const int n = mesh->numElements();
  double dNm = 0;
  for (int i = 0; i < n; ++i) {
    double Ni = 0;
    for (int nu = 0; nu < nc; ++nu) Ni += N_prev[(size_t)nu * n + i];
    double dNi = 0;
    for (int nu = 0; nu < nc; ++nu) dNi += std::fabs(dN[(size_t)nu * n + i]);
    dNm = jmax(dNm, dNi / Ni);
  }
  return dtFactor(dNm, c.target_throughput, c);
}

double Simulator::calculateDt(double dt, const rsg_dt_control& c, rsg_dt_factors* f) const {
  // :928-964
  double R = residualVolumeFactor(c);
  double NR = dtFactor(pressureIterations, c.target_nonlinear_iterations, c);
  double T = throughputFactor(c);
  double dt_R = dt * R, dt_NR = dt * NR, dt_T = dt * T;
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
  return st == ST_NOT_CONVERGED_ITERATIONS || st == ST_NOT_CONVERGED_DIVERGENCE || st == ST_NOT_CONVERGED_BREAKDOWN ||
         st == ST_NONPOSITIVE_PRESSURE || st == ST_NEGATIVE_MOLES || st == ST_NEWTON_NOT_CONVERGED;
}

int Simulator::stepTo(double endTime, const rsg_dt_control& c, double& dt, rsg_step_to_info* info) {
  // TimeStepper.stepTo (:58-102) with adjustDtForReporting (:117-128)
  rsg_step_to_info loc{};
  rsg_step_to_info& in = info ? *info : loc;
  in = rsg_step_to_info{};
  while (time < endTime) {
    if (dt + time > endTime) dt = endTime - time;
    while (true) {
      rsg_step_info si{};
      int st = 0;
      try {
        step(dt, &si);
      } catch (Failure& f) {
        st = f.status;
        if (!solver_failure(st)) throw;
      }
      in.status = st;
      if (st == 0) {
        in.steps++;
        in.newton_iterations += si.newton_iterations;
        in.linear_iterations += si.linear_iterations;
        break;
      }
      if (!(dt > c.dt_min)) {
        in.time = time;
        return st;  // timestep cannot be further reduced
      }
      retract();
      in.retries++;
      double factor = std::min(1. / 2., throughputFactor(c));
      dt = std::min(std::max(dt * factor, c.dt_min), c.dt_max);
    }
    dt = calculateDt(dt, c, nullptr);
  }
  in.time = time;
  return 0;
}

}  // namespace orc
