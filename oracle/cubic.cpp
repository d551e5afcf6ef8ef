// Oracle (test infrastructure only): restatement of RS's cubic equation of
// state and flash (rs/src/no/uib/cipr/rs/fluid/CubicEquationOfState.java)
// with the cubic root solver of util/CubicEquation.java and the water phase of
// fluid/WaterEquationOfState.java:72-129.  Every expression keeps the Java
// operand order (the build disables contraction).  Two departures, both shared
// with the GPU code: Composition totals are plain sums (the Java keeps a
// running total), and the flash and Rachford-Rice loops stop with a failure
// after a bounded number of iterations where the Java loops are unbounded.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "physics.hpp"

namespace orc {

namespace {

constexpr int NC = RSG_MAX_COMPONENTS;
constexpr double RGAS = 8.3145;  // util/Constants.R

double jmax(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  return a >= b ? a : b;
}

double signum(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : x); }

// CubicEquation.solve (util/CubicEquation.java:66-99)
void cubic_roots(double a0, double a1, double a2, double& zMin, double& zMid, double& zMax) {
  double Q = (3 * a1 - a2 * a2) / 9.;
  double R = (9 * a1 * a2 - 27 * a0 - 2 * a2 * a2 * a2) / 54.;
  double D = Q * Q * Q + R * R;
  if (D > 0 || Q == 0) {
    double Sarg = R + std::sqrt(D);
    double Targ = R - std::sqrt(D);
    double S = signum(Sarg) * std::pow(std::fabs(Sarg), 1. / 3.);
    double T = signum(Targ) * std::pow(std::fabs(Targ), 1. / 3.);
    zMin = zMid = zMax = -a2 / 3. + S + T;
  } else {
    double theta = std::acos(R / std::sqrt(-Q * Q * Q));
    double factor = 2 * std::sqrt(-Q);
    double z[3];
    z[0] = factor * std::cos(theta / 3.) - a2 / 3;
    z[1] = factor * std::cos((theta + 2 * M_PI) / 3.) - a2 / 3;
    z[2] = factor * std::cos((theta + 4 * M_PI) / 3.) - a2 / 3;
    std::sort(z, z + 3);
    zMin = z[0];
    zMid = z[1];
    zMax = z[2];
  }
}

struct Comp {  // fluid/Composition with a plain-sum total
  double N[NC] = {0};
  int nc = 0;
  double NT() const {
    double s = 0;
    for (int i = 0; i < nc; ++i) s += N[i];
    return s;
  }
  double x(int i) const {
    double t = NT();
    return t > 0 ? N[i] / t : 0;
  }
};

struct Cubic {
  const rsg_cubic_fluid& f;
  int nc;
  double d1, d2, OmegaA, OmegaB;
  double mi[NC], bi[NC], sqrtM[NC], zeta_inv[NC];
  // ComponentParameters.update(T)
  double ai[NC], daidT[NC], aij[NC][NC], daijdT[NC][NC];

  explicit Cubic(const rsg_cubic_fluid& fl) : f(fl), nc(fl.nc) {
    // EOS enum (:48-79) and ComponentParameters() (:405-417)
    if (f.eos == RSG_EOS_PR) {
      d1 = -(1 + std::sqrt(2.));
      d2 = -(1 - std::sqrt(2.));
      OmegaA = 0.457235529;
      OmegaB = 0.077796074;
    } else {
      d1 = -1;
      d2 = 0;
      OmegaA = 0.42748;
      OmegaB = 0.08664;
    }
    for (int i = 1; i < nc; ++i) {
      double w = f.omega[i];
      if (f.eos == RSG_EOS_PR)
        mi[i] = w > 0.49 ? 0.379642 + 1.48503 * w - 0.164423 * w * w + 0.016666 * w * w * w
                         : 0.37464 + 1.53226 * w - 0.26992 * w * w;
      else
        mi[i] = 0.48508 + 1.55171 * w - 0.15613 * w * w;
      bi[i] = OmegaB * RGAS * f.Tc[i] / f.pc[i];
      // HydrocarbonViscosity() (:1247-1257)
      sqrtM[i] = std::sqrt(f.Mw[i]);
      zeta_inv[i] = sqrtM[i] * std::pow(f.pc[i], 2. / 3) / std::pow(f.Tc[i], 1. / 6);
    }
  }

  void update(double T) {
    // ComponentParameters.update (:419-447)
    for (int i = 1; i < nc; ++i) {
      double Tci = f.Tc[i], pci = f.pc[i];
      double Tr = T / Tci;
      double alpha = 1 + mi[i] * (1 - std::sqrt(Tr));
      double dalphadT = -(mi[i] / 2) * (1 / std::sqrt(Tci * T));
      ai[i] = OmegaA * RGAS * RGAS * Tci * Tci * alpha * alpha / pci;
      daidT[i] = 2 * (ai[i] / alpha) * dalphadT;
    }
    for (int i = 1; i < nc; ++i)
      for (int j = 1; j < nc; ++j) {
        double dij = f.bic[i * NC + j];
        double sqr_ai_aj = std::sqrt(ai[i] * ai[j]);
        aij[i][j] = (1 - dij) * sqr_ai_aj;
        daijdT[i][j] = (1 - dij) * (ai[j] * daidT[i] + ai[i] * daidT[j]) / (2 * sqr_ai_aj);
      }
  }
};

struct PhaseParams {  // CubicEquationOfState.PhaseParameters (:452-741)
  bool oil;
  double a, b, dadT, A, B, dAdp, dBdp, dAdT, dBdT;
  double dadN[NC], dbdN[NC], dAdN[NC], dBdN[NC];
  double Z, dZdp, dZdT, dZdN[NC];
  double f[NC], phi[NC], dfdp[NC], dfdT[NC], dfdN[NC][NC];

  void parameters(const Cubic& c, double p, double T, const Comp& N) {
    // :529-582
    a = b = dadT = 0;
    for (int i = 1; i < c.nc; ++i) {
      double Ci = N.x(i);
      b += Ci * c.bi[i];
      for (int j = 1; j < c.nc; ++j) {
        double Cj = N.x(j);
        a += Ci * Cj * c.aij[i][j];
        dadT += Ci * Cj * c.daijdT[i][j];
      }
    }
    double Nl = N.NT();
    for (int i = 1; i < c.nc; ++i) {
      dbdN[i] = (c.bi[i] - b) / Nl;
      double sum = 0;
      for (int j = 1; j < c.nc; ++j) sum += N.x(j) * c.aij[i][j];
      dadN[i] = 2 * (sum - a) / Nl;
    }
    const double RT = RGAS * T;
    A = p * a / (RT * RT);
    B = p * b / RT;
    dAdp = A / p;
    dBdp = B / p;
    dAdT = -2 * (A / T) + (A / a) * dadT;
    dBdT = -B / T;
    for (int i = 1; i < c.nc; ++i) {
      dAdN[i] = (A / a) * dadN[i];
      dBdN[i] = (B / b) * dbdN[i];
    }
  }

  double dZdX(const Cubic& c, double a1, double a2, double dAdX, double dBdX) const {
    // :649-660
    double da0dX = -dAdX * B - dBdX * (A + B * (2 + 3 * B) * c.d1 * c.d2);
    double da1dX = dAdX + dBdX * ((1 + 2 * B) * (c.d1 + c.d2) + 2 * c.d1 * c.d2 * B);
    double da2dX = -dBdX * (1 + c.d1 + c.d2);
    return -(da2dX * Z * Z + da1dX * Z + da0dX) / (3 * Z * Z + 2 * a2 * Z + a1);
  }

  void compressibility(const Cubic& c) {
    // :587-616
    double a0 = -A * B - (B * B) * (1 + B) * c.d1 * c.d2;
    double a1 = A + B * (1 + B) * (c.d1 + c.d2) + c.d1 * c.d2 * B * B;
    double a2 = -1 - B * (1 + c.d1 + c.d2);
    double zMin, zMid, zMax;
    cubic_roots(a0, a1, a2, zMin, zMid, zMax);
    if (oil) {
      Z = zMin;
      if (Z < 0) {
        Z = zMid;
        if (Z < 0) Z = zMax;
      }
    } else {
      Z = zMax;
    }
    if (!(Z > 0)) throw Failure(ST_PHYSICS, "Z = " + std::to_string(Z) + " <= 0");
    dZdp = dZdX(c, a1, a2, dAdp, dBdp);
    dZdT = dZdX(c, a1, a2, dAdT, dBdT);
    for (int i = 1; i < c.nc; ++i) dZdN[i] = dZdX(c, a1, a2, dAdN[i], dBdN[i]);
  }

  void translate(const Cubic& c, double p, double T, const Comp& N) {
    // applyVolumeTranslation (:621-644)
    const double RT = RGAS * T;
    double Nl = N.NT();
    double shift = 0;
    for (int i = 1; i < c.nc; ++i) {
      double ci = c.f.shift[i] * c.bi[i];
      shift += N.x(i) * ci;
    }
    Z -= (p / RT) * shift;
    dZdp -= (1 / RT) * shift;
    dZdT -= (p / (RT * T)) * shift;
    for (int i = 1; i < c.nc; ++i) {
      double ci = c.f.shift[i] * c.bi[i];
      dZdN[i] -= (p / RT) * (ci - shift) / Nl;
    }
  }

  double dphidX(const Cubic& c, double y, double w, double lnw, double v, double ph, double alpha, double beta,
                double dAdX, double dBdX, double dZdX_, double dalphadX, double dbetadX) const {
    // :728-741
    double dydX = (dbetadX * (Z - 1) + beta * dZdX_) * y - (y / (Z - B)) * (dZdX_ - dBdX);
    double dvdX = (dAdX * (alpha - beta) + A * (dalphadX - dbetadX)) / ((c.d2 - c.d1) * B) - (v / B) * dBdX;
    double dwdX = (dZdX_ - c.d2 * dBdX - w * (dZdX_ - c.d1 * dBdX)) / (Z - c.d1 * B);
    return dydX * (ph / y) + ph * (dvdX * lnw + (v / w) * dwdX);
  }

  void fugacities(const Cubic& c, double p, const Comp& N) {
    // :665-721
    double Nl = N.NT();
    double w = (Z - c.d2 * B) / (Z - c.d1 * B);
    double lnw = std::log(w);
    for (int i = 1; i < c.nc; ++i) {
      double alpha = 0;
      for (int j = 1; j < c.nc; ++j) {
        double Cj = N.x(j);
        alpha += Cj * c.aij[i][j];
      }
      alpha *= (2 / a);
      double beta = c.bi[i] / b;
      double y = std::exp(beta * (Z - 1)) / (Z - B);
      double v = A * (alpha - beta) / ((c.d2 - c.d1) * B);
      phi[i] = y * std::pow(w, v);
      double Ci = N.x(i);
      f[i] = p * Ci * phi[i];
      double dalphadT = -(alpha / a) * dadT;
      for (int j = 1; j < c.nc; ++j) {
        double Cj = N.x(j);
        dalphadT += (2 / a) * Cj * c.daijdT[i][j];
      }
      double dphidp = dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdp, dBdp, dZdp, 0, 0);
      double dphidT = dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdT, dBdT, dZdT, dalphadT, 0);
      dfdp[i] = f[i] / p + (f[i] / phi[i]) * dphidp;
      dfdT[i] = (f[i] / phi[i]) * dphidT;
      for (int j = 1; j < c.nc; ++j) {
        double dalphadN = -(alpha / a) * dadN[j] + (2 / a) * c.aij[i][j] / Nl - alpha / Nl;
        double dbetadN = -(beta / b) * dbdN[j];
        double dphidN = dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdN[j], dBdN[j], dZdN[j], dalphadN, dbetadN);
        double delta = (i == j) ? 1 : 0;
        double div = (Ci == 0) ? 1 : Ci;
        dfdN[i][j] = (f[i] / div) * (delta - Ci) / Nl + (f[i] / phi[i]) * dphidN;
      }
    }
  }

  void calculate(const Cubic& c, double p, double T, const Comp& N) {
    parameters(c, p, T, N);
    compressibility(c);
    translate(c, p, T, N);
    fugacities(c, p, N);
  }
};

constexpr int RR_MAX_ITERATIONS = 200;

struct Flash {  // CubicEquationOfState.Flash (:753-1212)
  Cubic& c;
  PhaseParams& op;
  PhaseParams& gp;
  double C[NC], K[NC], r[NC];
  double dNodp[NC], dNodT[NC], dNodN[NC][NC];
  int iterations = 0;
  Flash(Cubic& cc, PhaseParams& o, PhaseParams& g) : c(cc), op(o), gp(g) {}

  double fRR(double L) const {
    double f = 0;
    for (int i = 1; i < c.nc; ++i) {
      double nom = (K[i] - 1) * C[i];
      double denom = L + (1 - L) * K[i];
      if (denom != 0) f += nom / denom;
    }
    return f;
  }
  double dfdL(double L) const {
    double d = 0;
    for (int i = 1; i < c.nc; ++i) {
      double factor = (K[i] - 1) / (L + (1 - L) * K[i]);
      d += factor * factor * C[i];
    }
    return d;
  }
  double rachfordRice(double L) const {
    // solveRachfordRice (:1122-1165)
    double f0 = fRR(0);
    if (f0 >= 0) return 0;
    double f1 = fRR(1);
    if (f1 <= 0) return 1;
    double f = fRR(L);
    int it = 0;
    while (std::fabs(f) > 1e-12) {
      if (++it > RR_MAX_ITERATIONS) throw Failure(ST_PHYSICS, "Rachford-Rice iteration did not converge");
      double d = dfdL(L);
      double alpha = 1;
      if (f > 0) {
        double alpha0 = L * (d / f);
        if (alpha0 < alpha) alpha = alpha0;
      } else {
        double alpha1 = (L - 1) * (d / f);
        if (alpha1 < alpha) alpha = alpha1;
      }
      L -= alpha * f / d;
      f = fRR(L);
    }
    return L;
  }
  void setOilGas(const Comp& N, double L, Comp& oil, Comp& gas) const {
    // setOilGasComposition (:1102-1113)
    double NHC = N.NT() - N.N[0];
    double No = L * NHC, Ng = (1 - L) * NHC;
    for (int i = 1; i < c.nc; ++i) {
      double Co = C[i] / (L + (1 - L) * K[i]);
      oil.N[i] = Co * No;
      gas.N[i] = K[i] * Co * Ng;
    }
  }
  double residual() {
    // calculateResidual (:975-982), infinity norm
    double m = 0;
    for (int i = 1; i < c.nc; ++i) {
      r[i - 1] = op.f[i] - gp.f[i];
      m = jmax(m, std::fabs(r[i - 1]));
    }
    return m;
  }
  void flash(double p, double T, const Comp& N, Comp& oil, Comp& gas) {
    // flash (:871-973)
    const int m = c.nc - 1;
    double NHC = N.NT() - N.N[0];
    for (int i = 1; i < c.nc; ++i) C[i] = N.N[i] / NHC;  // setHydrocarbonFractions
    double res = 1.7976931348623157e308;
    double L = 0.5;
    if (oil.NT() == 0 || gas.NT() == 0) {
      for (int i = 1; i < c.nc; ++i) {  // calculateInitialK (:1203-1211)
        double Tri = c.f.Tc[i] / T;
        double pri = c.f.pc[i] / p;
        K[i] = pri * std::exp(5.373 * (1 + c.f.omega[i]) * (1 - Tri));
      }
    } else {
      op.calculate(c, p, T, oil);
      gp.calculate(c, p, T, gas);
      for (int i = 1; i < c.nc; ++i) K[i] = op.phi[i] / gp.phi[i];
      L = oil.NT() / (oil.NT() + gas.NT());
    }
    iterations = 0;
    do {
      if (++iterations > c.f.flash_max_iterations) throw Failure(ST_PHYSICS, "flash did not converge");
      if (res > c.f.flash_criteria) {
        L = rachfordRice(L);
        setOilGas(N, L, oil, gas);
        if (L > 0) op.calculate(c, p, T, oil);
        if (L < 1) gp.calculate(c, p, T, gas);
        if (L == 0) {
          for (int i = 0; i < c.nc; ++i) oil.N[i] = 0;
          break;
        } else if (L == 1) {
          for (int i = 0; i < c.nc; ++i) gas.N[i] = 0;
          break;
        }
        for (int i = 1; i < c.nc; ++i) K[i] = op.phi[i] / gp.phi[i];
      } else {
        // buildJacobian (:990-1012); F x = -r by DenseLU
        double F[NC * NC] = {0}, x[NC];
        for (int i = 1; i < c.nc; ++i) {
          double Ci = N.x(i);
          if (Ci == 0) {
            F[(i - 1) + (i - 1) * m] = 1;
            continue;
          }
          for (int j = 1; j < c.nc; ++j) F[(i - 1) + (j - 1) * m] = op.dfdN[i][j] + gp.dfdN[i][j];
        }
        for (int i = 0; i < m; ++i) x[i] = -1 * r[i];
        int piv[NC];
        if (dgetf2(m, F, m, piv) > 0) throw Failure(ST_SINGULAR, "MatrixSingularException in the flash");
        dgetrs(false, m, F, m, piv, x);
        double alpha = 1;
        for (int i = 1; i < c.nc; ++i) {
          if (N.N[i] == 0) continue;
          double No = oil.N[i], Ng = gas.N[i];
          double dNo = x[i - 1];
          if (No + alpha * dNo < 0) alpha = -No / dNo;
          if (Ng - alpha * dNo < 0) alpha = Ng / dNo;
        }
        for (int i = 1; i < c.nc; ++i) {
          if (N.N[i] == 0) continue;
          double dNo = alpha * x[i - 1];
          oil.N[i] += dNo;
          gas.N[i] += -dNo;
        }
        op.calculate(c, p, T, oil);
        gp.calculate(c, p, T, gas);
      }
    } while ((res = residual()) > c.f.flash_tolerance);
  }
  void molarMassDerivatives(const Comp& N) {
    // calculateMolarMassDerivatives (:1022-1087): F X = R, R with nc+1 columns
    const int m = c.nc - 1, pi = c.nc - 1, Ti = pi + 1;
    double F[NC * NC] = {0}, R[NC * (NC + 1)] = {0};
    for (int i = 1; i < c.nc; ++i) {
      if (N.N[i] == 0) {
        F[(i - 1) + (i - 1) * m] = 1;
        continue;
      }
      R[(i - 1) + pi * m] = gp.dfdp[i] - op.dfdp[i];
      R[(i - 1) + Ti * m] = gp.dfdT[i] - op.dfdT[i];
      for (int j = 1; j < c.nc; ++j) {
        if (N.N[j] == 0) continue;
        F[(i - 1) + (j - 1) * m] = op.dfdN[i][j] + gp.dfdN[i][j];
        R[(i - 1) + (j - 1) * m] = gp.dfdN[i][j];
      }
    }
    int piv[NC];
    if (dgetf2(m, F, m, piv) > 0) throw Failure(ST_SINGULAR, "MatrixSingularException in the molar derivatives");
    for (int col = 0; col < c.nc + 1; ++col) dgetrs(false, m, F, m, piv, R + col * m);
    for (int i = 1; i < c.nc; ++i) {
      dNodp[i] = R[(i - 1) + pi * m];
      dNodT[i] = R[(i - 1) + Ti * m];
      for (int j = 1; j < c.nc; ++j) dNodN[i][j] = R[(i - 1) + (j - 1) * m];
    }
  }
};

void set_present(EOSData& d, bool exists, int nc) {
  // EquationOfStateData.setPresent (:107-121)
  d.present = exists;
  if (!exists) {
    d.V = d.xi = d.dVdp = d.dVdT = d.h = d.dhdT = d.mu = 0;
    for (int i = 0; i < nc; ++i) d.N[i] = d.dVdN[i] = 0;
  }
}

double viscosity(const Cubic& c, double T, const Comp& N, double xi) {
  // HydrocarbonViscosity.calculateViscosity (:1289-1337)
  const double c1 = 3.4e-4, c2 = 1.778e-4, c3 = 4.58, c4 = 1.67;
  const double e1 = 0.94, e2 = 0.625;
  const double Tdiv = 1.5;
  double Vcl = 0, Tcl = 0, Ml = 0, pcl = 0, M2l = 0, musl = 0;
  for (int i = 1; i < c.nc; ++i) {
    double C = N.x(i);
    double M = c.f.Mw[i], Tc = c.f.Tc[i], pc = c.f.pc[i], Vc = c.f.Vc[i];
    Vcl += C * Vc;
    Tcl += C * Tc;
    Ml += C * M;
    pcl += C * pc;
    M2l += C * c.sqrtM[i];
    double mui = 0;
    double Tr = T / Tc;
    if (Tr > Tdiv) mui = c1 * std::pow(Tr, e1);
    else mui = c2 * std::pow(c3 * Tr - c4, e2);
    mui *= c.zeta_inv[i];
    musl += C * mui * c.sqrtM[i];
  }
  musl /= M2l;
  double zinv = std::sqrt(Ml) * std::pow(pcl, 2. / 3) / std::pow(Tcl, 1. / 6);
  double xir = xi * Vcl;
  const double* a = c.f.lbc;
  double chi = a[0] + xir * (a[1] + xir * (a[2] + xir * (a[3] + xir * a[4])));
  double mu = musl + zinv * (chi * chi * chi * chi - 1e-4);
  if (mu != mu) return 0;
  return mu * 1e-3;
}

}  // namespace

// CubicEquationOfState.calculatePhaseState (:188-266) with the water phase of
// WaterEquationOfState.calculatePhaseState (:72-129); ph = {water, oil, gas}.
int cubic_phase_state(const rsg_cubic_fluid& fl, const Function& wden, const Function& wvis, double p, double T,
                      const double* Nin, EOSData* ph) {
  const int nc = fl.nc;
  Comp N;
  N.nc = nc;
  for (int i = 0; i < nc; ++i) N.N[i] = Nin[i];
  // water
  {
    EOSData& w = ph[WATER];
    double Nw = N.N[0];
    double pT[2] = {p, T};
    if (Nw > 0) {
      set_present(w, true, nc);
      double xiw = wden.get(pT);
      double Vw = Nw / xiw;
      w.xi = xiw;
      w.V = Vw;
      w.N[0] = Nw;
      double dxiw_dp = wden.deriv(0, pT);
      double dxiw_dT = wden.deriv(1, pT);
      if (dxiw_dp < 0) throw Failure(ST_PHYSICS, "Water molar density pressure derivative cannot be negative");
      w.dVdp = -(Vw / xiw) * dxiw_dp;
      w.dVdT = -(Vw / xiw) * dxiw_dT;
      w.dVdN[0] = 1 / xiw;
      w.mu = wvis.get(pT);
    } else {
      set_present(w, false, nc);
    }
  }
  Cubic c(fl);
  c.update(T);
  PhaseParams op{}, gp{};
  op.oil = true;
  gp.oil = false;
  Comp oil, gas;
  oil.nc = gas.nc = nc;
  for (int i = 0; i < nc; ++i) {
    oil.N[i] = ph[OIL].N[i];
    gas.N[i] = ph[GAS].N[i];
  }
  Flash fl_(c, op, gp);
  fl_.flash(p, T, N, oil, gas);
  for (int i = 1; i < nc; ++i)
    if (N.N[i] == 0) {
      oil.N[i] = 0;
      gas.N[i] = 0;
    }
  EOSData& od = ph[OIL];
  EOSData& gd = ph[GAS];
  set_present(od, oil.NT() > 0, nc);
  set_present(gd, gas.NT() > 0, nc);
  if (od.present)
    for (int i = 0; i < nc; ++i) od.N[i] = oil.N[i];
  if (gd.present)
    for (int i = 0; i < nc; ++i) gd.N[i] = gas.N[i];
  const double RT = RGAS * T;
  auto props = [&](PhaseParams& pp, EOSData& d, const Comp& comp) {
    // calculatePhaseProperties (:268-279)
    double V = pp.Z * comp.NT() * RT / p;
    d.V = V;
    d.xi = p / (pp.Z * RT);
  };
  if (od.present) props(op, od, oil);
  if (gd.present) props(gp, gd, gas);
  auto single = [&](PhaseParams& pp, EOSData& d, const Comp& comp) {
    // calculateVolumeDerivativesSinglePhase (:281-300)
    double V = d.V, Z = pp.Z;
    d.dVdp = (V / Z) * pp.dZdp - V / p;
    d.dVdT = (V / Z) * pp.dZdT + V / T;
    double Nl = comp.NT();
    for (int i = 1; i < nc; ++i) d.dVdN[i] = (V / Z) * pp.dZdN[i] + V / Nl;
  };
  if (od.present && gd.present) {
    // calculateVolumeDerivativesTwoPhase (:302-385)
    fl_.molarMassDerivatives(N);
    double Vo = od.V, Vg = gd.V, Zo = op.Z, Zg = gp.Z;
    double dZodp = op.dZdp, dZgdp = gp.dZdp, dZodT = op.dZdT, dZgdT = gp.dZdT;
    double dNodp = 0, dNodT = 0;
    for (int i = 1; i < nc; ++i) {
      dNodp += fl_.dNodp[i];
      dNodT += fl_.dNodT[i];
      dZodp += op.dZdN[i] * fl_.dNodp[i];
      dZgdp -= gp.dZdN[i] * fl_.dNodp[i];
      dZodT += op.dZdN[i] * fl_.dNodT[i];
      dZgdT -= gp.dZdN[i] * fl_.dNodT[i];
    }
    double dNgdp = -dNodp, dNgdT = -dNodT;
    double No = oil.NT(), Ng = gas.NT();
    od.dVdp = (Vo / Zo) * dZodp + (Vo / No) * dNodp - Vo / p;
    gd.dVdp = (Vg / Zg) * dZgdp + (Vg / Ng) * dNgdp - Vg / p;
    od.dVdT = (Vo / Zo) * dZodT + (Vo / No) * dNodT + Vo / T;
    gd.dVdT = (Vg / Zg) * dZgdT + (Vg / Ng) * dNgdT + Vg / T;
    for (int i = 1; i < nc; ++i) {
      double dVodNi = 0, dVgdNi = 0;
      for (int j = 1; j < nc; ++j) {
        if (N.N[j] == 0) continue;
        double dNodNi = fl_.dNodN[j][i];
        double dNgdNi = -dNodNi;
        if (i == j) dNgdNi++;
        double dZodN = op.dZdN[j], dZgdN = gp.dZdN[j];
        dVodNi += ((Vo / Zo) * dZodN + Vo / No) * dNodNi;
        dVgdNi += ((Vg / Zg) * dZgdN + Vg / Ng) * dNgdNi;
      }
      od.dVdN[i] = dVodNi;
      gd.dVdN[i] = dVgdNi;
    }
  } else if (od.present) {
    single(op, od, oil);
  } else if (gd.present) {
    single(gp, gd, gas);
  }
  if (od.present) od.mu = viscosity(c, T, oil, od.xi);
  if (gd.present) gd.mu = viscosity(c, T, gas, gd.xi);
  return fl_.iterations;
}

void cubic_roots_kat(double a0, double a1, double a2, double* z) { cubic_roots(a0, a1, a2, z[0], z[1], z[2]); }

}  // namespace orc
