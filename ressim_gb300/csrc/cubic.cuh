// Cubic equation of state and isothermal flash, one cell per thread
// (rs/src/no/uib/cipr/rs/fluid/CubicEquationOfState.java, with the root
// solver of util/CubicEquation.java).  Included inside sim.cu's unnamed
// namespace, after DFunc/f_eval.  Expressions keep the Java operand order;
// Composition totals are plain sums, and the flash and Rachford-Rice loops
// give up after a bounded number of iterations (the Java loops are unbounded).
#pragma once

constexpr double CUBIC_R = 8.3145;  // util/Constants.R
constexpr int RR_MAX_ITERATIONS = 200;

enum { CUBIC_OK = 0, CUBIC_Z = 1, CUBIC_SINGULAR = 2, CUBIC_RR = 3, CUBIC_FLASH = 4, CUBIC_WATER = 5 };

// Everything of the fluid that does not depend on the cell (host-computed:
// ComponentParameters(), HydrocarbonViscosity() and the EOS constants).
struct DCubic {
  int nc, eos, maxit;
  double d1, d2, OmegaA, OmegaB, criteria, tol;
  double Tc[NCM], pc[NCM], omega[NCM], Mw[NCM], Vc[NCM], s[NCM];
  double mi[NCM], bi[NCM], sqrtM[NCM], zeta_inv[NCM];
  double dij[NCM][NCM];
  double lbc[5];
  DFunc wden, wvis;
};

struct CComp {
  double N[NCM];
  __device__ double NT(int nc) const {
    double s = 0;
    for (int i = 0; i < nc; ++i) s += N[i];
    return s;
  }
  __device__ double x(int nc, int i) const {
    const double t = NT(nc);
    return t > 0 ? N[i] / t : 0;
  }
};

struct CTemp {  // ComponentParameters.update(T)
  double ai[NCM], daidT[NCM], aij[NCM][NCM], daijdT[NCM][NCM];
};

__device__ double jmaxd(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  return a >= b ? a : b;
}

__device__ void cubic_update(const DCubic& c, double T, CTemp& t) {
  for (int i = 1; i < c.nc; ++i) {
    const double Tci = c.Tc[i], pci = c.pc[i];
    const double Tr = T / Tci;
    const double alpha = 1 + c.mi[i] * (1 - sqrt(Tr));
    const double dalphadT = -(c.mi[i] / 2) * (1 / sqrt(Tci * T));
    t.ai[i] = c.OmegaA * CUBIC_R * CUBIC_R * Tci * Tci * alpha * alpha / pci;
    t.daidT[i] = 2 * (t.ai[i] / alpha) * dalphadT;
  }
  for (int i = 1; i < c.nc; ++i)
    for (int j = 1; j < c.nc; ++j) {
      const double sqr_ai_aj = sqrt(t.ai[i] * t.ai[j]);
      t.aij[i][j] = (1 - c.dij[i][j]) * sqr_ai_aj;
      t.daijdT[i][j] = (1 - c.dij[i][j]) * (t.ai[j] * t.daidT[i] + t.ai[i] * t.daidT[j]) / (2 * sqr_ai_aj);
    }
}

__device__ void cubic_solve(double a0, double a1, double a2, double* z) {
  const double Q = (3 * a1 - a2 * a2) / 9.;
  const double R = (9 * a1 * a2 - 27 * a0 - 2 * a2 * a2 * a2) / 54.;
  const double D = Q * Q * Q + R * R;
  if (D > 0 || Q == 0) {
    const double Sarg = R + sqrt(D);
    const double Targ = R - sqrt(D);
    const double sS = Sarg > 0 ? 1.0 : (Sarg < 0 ? -1.0 : Sarg);
    const double sT = Targ > 0 ? 1.0 : (Targ < 0 ? -1.0 : Targ);
    const double S = sS * pow(fabs(Sarg), 1. / 3.);
    const double Tt = sT * pow(fabs(Targ), 1. / 3.);
    z[0] = z[1] = z[2] = -a2 / 3. + S + Tt;
    return;
  }
  const double theta = acos(R / sqrt(-Q * Q * Q));
  const double factor = 2 * sqrt(-Q);
  z[0] = factor * cos(theta / 3.) - a2 / 3;
  z[1] = factor * cos((theta + 2 * M_PI) / 3.) - a2 / 3;
  z[2] = factor * cos((theta + 4 * M_PI) / 3.) - a2 / 3;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2 - a; ++b)
      if (z[b] > z[b + 1]) {
        const double t = z[b];
        z[b] = z[b + 1];
        z[b + 1] = t;
      }
}

struct CPhase {  // PhaseParameters
  bool oil;
  double a, b, dadT, A, B, dAdp, dBdp, dAdT, dBdT;
  double dadN[NCM], dbdN[NCM], dAdN[NCM], dBdN[NCM];
  double Z, dZdp, dZdT, dZdN[NCM];
  double f[NCM], phi[NCM], dfdp[NCM], dfdT[NCM], dfdN[NCM][NCM];

  __device__ double dZdX(const DCubic& c, double a1, double a2, double dAdX, double dBdX) const {
    const double da0dX = -dAdX * B - dBdX * (A + B * (2 + 3 * B) * c.d1 * c.d2);
    const double da1dX = dAdX + dBdX * ((1 + 2 * B) * (c.d1 + c.d2) + 2 * c.d1 * c.d2 * B);
    const double da2dX = -dBdX * (1 + c.d1 + c.d2);
    return -(da2dX * Z * Z + da1dX * Z + da0dX) / (3 * Z * Z + 2 * a2 * Z + a1);
  }

  __device__ double dphidX(const DCubic& c, double y, double w, double lnw, double v, double ph, double alpha,
                           double beta, double dAdX, double dBdX, double dZdX_, double dalphadX,
                           double dbetadX) const {
    const double dydX = (dbetadX * (Z - 1) + beta * dZdX_) * y - (y / (Z - B)) * (dZdX_ - dBdX);
    const double dvdX = (dAdX * (alpha - beta) + A * (dalphadX - dbetadX)) / ((c.d2 - c.d1) * B) - (v / B) * dBdX;
    const double dwdX = (dZdX_ - c.d2 * dBdX - w * (dZdX_ - c.d1 * dBdX)) / (Z - c.d1 * B);
    return dydX * (ph / y) + ph * (dvdX * lnw + (v / w) * dwdX);
  }

  // calculate(p, T, N): phase parameters, compressibility, volume shift,
  // fugacities and their derivatives
  __device__ int calculate(const DCubic& c, const CTemp& t, double p, double T, const CComp& N) {
    const int nc = c.nc;
    a = b = dadT = 0;
    for (int i = 1; i < nc; ++i) {
      const double Ci = N.x(nc, i);
      b += Ci * c.bi[i];
      for (int j = 1; j < nc; ++j) {
        const double Cj = N.x(nc, j);
        a += Ci * Cj * t.aij[i][j];
        dadT += Ci * Cj * t.daijdT[i][j];
      }
    }
    const double Nl = N.NT(nc);
    for (int i = 1; i < nc; ++i) {
      dbdN[i] = (c.bi[i] - b) / Nl;
      double sum = 0;
      for (int j = 1; j < nc; ++j) sum += N.x(nc, j) * t.aij[i][j];
      dadN[i] = 2 * (sum - a) / Nl;
    }
    const double RT = CUBIC_R * T;
    A = p * a / (RT * RT);
    B = p * b / RT;
    dAdp = A / p;
    dBdp = B / p;
    dAdT = -2 * (A / T) + (A / a) * dadT;
    dBdT = -B / T;
    for (int i = 1; i < nc; ++i) {
      dAdN[i] = (A / a) * dadN[i];
      dBdN[i] = (B / b) * dbdN[i];
    }
    // calculatePhaseCompressibility
    const double a0 = -A * B - (B * B) * (1 + B) * c.d1 * c.d2;
    const double a1 = A + B * (1 + B) * (c.d1 + c.d2) + c.d1 * c.d2 * B * B;
    const double a2 = -1 - B * (1 + c.d1 + c.d2);
    double z[3];
    cubic_solve(a0, a1, a2, z);
    if (oil) {
      Z = z[0];
      if (Z < 0) {
        Z = z[1];
        if (Z < 0) Z = z[2];
      }
    } else {
      Z = z[2];
    }
    if (!(Z > 0)) return CUBIC_Z;
    dZdp = dZdX(c, a1, a2, dAdp, dBdp);
    dZdT = dZdX(c, a1, a2, dAdT, dBdT);
    for (int i = 1; i < nc; ++i) dZdN[i] = dZdX(c, a1, a2, dAdN[i], dBdN[i]);
    // applyVolumeTranslation
    double shift = 0;
    for (int i = 1; i < nc; ++i) {
      const double ci = c.s[i] * c.bi[i];
      shift += N.x(nc, i) * ci;
    }
    Z -= (p / RT) * shift;
    dZdp -= (1 / RT) * shift;
    dZdT -= (p / (RT * T)) * shift;
    for (int i = 1; i < nc; ++i) {
      const double ci = c.s[i] * c.bi[i];
      dZdN[i] -= (p / RT) * (ci - shift) / Nl;
    }
    // calculateFugacities
    const double w = (Z - c.d2 * B) / (Z - c.d1 * B);
    const double lnw = log(w);
    for (int i = 1; i < nc; ++i) {
      double alpha = 0;
      for (int j = 1; j < nc; ++j) {
        const double Cj = N.x(nc, j);
        alpha += Cj * t.aij[i][j];
      }
      alpha *= (2 / a);
      const double beta = c.bi[i] / b;
      const double y = exp(beta * (Z - 1)) / (Z - B);
      const double v = A * (alpha - beta) / ((c.d2 - c.d1) * B);
      phi[i] = y * pow(w, v);
      const double Ci = N.x(nc, i);
      f[i] = p * Ci * phi[i];
      double dalphadT = -(alpha / a) * dadT;
      for (int j = 1; j < nc; ++j) {
        const double Cj = N.x(nc, j);
        dalphadT += (2 / a) * Cj * t.daijdT[i][j];
      }
      const double dphidp = dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdp, dBdp, dZdp, 0, 0);
      const double dphidT = dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdT, dBdT, dZdT, dalphadT, 0);
      dfdp[i] = f[i] / p + (f[i] / phi[i]) * dphidp;
      dfdT[i] = (f[i] / phi[i]) * dphidT;
      for (int j = 1; j < nc; ++j) {
        const double dalphadN = -(alpha / a) * dadN[j] + (2 / a) * t.aij[i][j] / Nl - alpha / Nl;
        const double dbetadN = -(beta / b) * dbdN[j];
        const double dphidN =
            dphidX(c, y, w, lnw, v, phi[i], alpha, beta, dAdN[j], dBdN[j], dZdN[j], dalphadN, dbetadN);
        const double delta = (i == j) ? 1 : 0;
        const double div = (Ci == 0) ? 1 : Ci;
        dfdN[i][j] = (f[i] / div) * (delta - Ci) / Nl + (f[i] / phi[i]) * dphidN;
      }
    }
    return CUBIC_OK;
  }
};

// dgetf2 / dgetrs ('N') on an m x m column-major block (DenseLU)
__device__ int small_lu(int m, double* A, int* piv) {
  int info = 0;
  for (int j = 0; j < m; ++j) {
    int jp = j;
    double amax = fabs(A[j + j * m]);
    for (int i = j + 1; i < m; ++i) {
      const double v = fabs(A[i + j * m]);
      if (v > amax) {
        amax = v;
        jp = i;
      }
    }
    piv[j] = jp;
    if (A[jp + j * m] != 0.0) {
      if (jp != j)
        for (int q = 0; q < m; ++q) {
          const double t = A[j + q * m];
          A[j + q * m] = A[jp + q * m];
          A[jp + q * m] = t;
        }
      if (j < m - 1) {
        const double rp = 1.0 / A[j + j * m];
        for (int i = j + 1; i < m; ++i) A[i + j * m] *= rp;
      }
    } else if (info == 0) {
      info = j + 1;
    }
    if (j < m - 1)
      for (int q = j + 1; q < m; ++q) {
        const double yv = A[j + q * m];
        if (yv != 0.0) {
          const double temp = -1.0 * yv;
          for (int i = j + 1; i < m; ++i) A[i + q * m] += A[i + j * m] * temp;
        }
      }
  }
  return info;
}

__device__ void small_solve(int m, const double* A, const int* piv, double* b) {
  for (int j = 0; j < m; ++j)
    if (piv[j] != j) {
      const double t = b[j];
      b[j] = b[piv[j]];
      b[piv[j]] = t;
    }
  for (int k = 0; k < m; ++k)
    if (b[k] != 0.0)
      for (int i = k + 1; i < m; ++i) b[i] -= b[k] * A[i + k * m];
  for (int k = m - 1; k >= 0; --k)
    if (b[k] != 0.0) {
      b[k] = b[k] / A[k + k * m];
      for (int i = 0; i < k; ++i) b[i] -= b[k] * A[i + k * m];
    }
}

struct CFlash {
  double C[NCM], K[NCM], r[NCM];
  double dNodp[NCM], dNodT[NCM], dNodN[NCM][NCM];
  int iterations;

  __device__ double fRR(int nc, double L) const {
    double f = 0;
    for (int i = 1; i < nc; ++i) {
      const double nom = (K[i] - 1) * C[i];
      const double denom = L + (1 - L) * K[i];
      if (denom != 0) f += nom / denom;
    }
    return f;
  }
  __device__ double dfdL(int nc, double L) const {
    double d = 0;
    for (int i = 1; i < nc; ++i) {
      const double factor = (K[i] - 1) / (L + (1 - L) * K[i]);
      d += factor * factor * C[i];
    }
    return d;
  }
  // solveRachfordRice; returns false when it does not converge
  __device__ bool rachford_rice(int nc, double& L) const {
    const double f0 = fRR(nc, 0);
    if (f0 >= 0) {
      L = 0;
      return true;
    }
    const double f1 = fRR(nc, 1);
    if (f1 <= 0) {
      L = 1;
      return true;
    }
    double f = fRR(nc, L);
    int it = 0;
    while (fabs(f) > 1e-12) {
      if (++it > RR_MAX_ITERATIONS) return false;
      const double d = dfdL(nc, L);
      double alpha = 1;
      if (f > 0) {
        const double alpha0 = L * (d / f);
        if (alpha0 < alpha) alpha = alpha0;
      } else {
        const double alpha1 = (L - 1) * (d / f);
        if (alpha1 < alpha) alpha = alpha1;
      }
      L -= alpha * f / d;
      f = fRR(nc, L);
    }
    return true;
  }
  __device__ double residual(int nc, const CPhase& op, const CPhase& gp) {
    double m = 0;
    for (int i = 1; i < nc; ++i) {
      r[i - 1] = op.f[i] - gp.f[i];
      m = jmaxd(m, fabs(r[i - 1]));
    }
    return m;
  }

  __device__ int flash(const DCubic& c, const CTemp& t, double p, double T, const CComp& N, CComp& oil, CComp& gas,
                       CPhase& op, CPhase& gp) {
    const int nc = c.nc, m = nc - 1;
    const double NHC = N.NT(nc) - N.N[0];
    for (int i = 1; i < nc; ++i) C[i] = N.N[i] / NHC;
    double res = 1.7976931348623157e308;
    double L = 0.5;
    if (oil.NT(nc) == 0 || gas.NT(nc) == 0) {
      for (int i = 1; i < nc; ++i) {
        const double Tri = c.Tc[i] / T;
        const double pri = c.pc[i] / p;
        K[i] = pri * exp(5.373 * (1 + c.omega[i]) * (1 - Tri));
      }
    } else {
      int e = op.calculate(c, t, p, T, oil);
      if (e) return e;
      e = gp.calculate(c, t, p, T, gas);
      if (e) return e;
      for (int i = 1; i < nc; ++i) K[i] = op.phi[i] / gp.phi[i];
      L = oil.NT(nc) / (oil.NT(nc) + gas.NT(nc));
    }
    iterations = 0;
    do {
      if (++iterations > c.maxit) return CUBIC_FLASH;
      if (res > c.criteria) {
        if (!rachford_rice(nc, L)) return CUBIC_RR;
        const double NHC2 = N.NT(nc) - N.N[0];
        const double No = L * NHC2, Ng = (1 - L) * NHC2;
        for (int i = 1; i < nc; ++i) {
          const double Co = C[i] / (L + (1 - L) * K[i]);
          oil.N[i] = Co * No;
          gas.N[i] = K[i] * Co * Ng;
        }
        if (L > 0) {
          const int e = op.calculate(c, t, p, T, oil);
          if (e) return e;
        }
        if (L < 1) {
          const int e = gp.calculate(c, t, p, T, gas);
          if (e) return e;
        }
        if (L == 0) {
          for (int i = 0; i < nc; ++i) oil.N[i] = 0;
          break;
        } else if (L == 1) {
          for (int i = 0; i < nc; ++i) gas.N[i] = 0;
          break;
        }
        for (int i = 1; i < nc; ++i) K[i] = op.phi[i] / gp.phi[i];
      } else {
        double F[NCM * NCM], x[NCM];
        int piv[NCM];
        for (int q = 0; q < m * m; ++q) F[q] = 0;
        for (int i = 1; i < nc; ++i) {
          const double Ci = N.x(nc, i);
          if (Ci == 0) {
            F[(i - 1) + (i - 1) * m] = 1;
            continue;
          }
          for (int j = 1; j < nc; ++j) F[(i - 1) + (j - 1) * m] = op.dfdN[i][j] + gp.dfdN[i][j];
        }
        for (int i = 0; i < m; ++i) x[i] = -1 * r[i];
        if (small_lu(m, F, piv) > 0) return CUBIC_SINGULAR;
        small_solve(m, F, piv, x);
        double alpha = 1;
        for (int i = 1; i < nc; ++i) {
          if (N.N[i] == 0) continue;
          const double No = oil.N[i], Ng = gas.N[i];
          const double dNo = x[i - 1];
          if (No + alpha * dNo < 0) alpha = -No / dNo;
          if (Ng - alpha * dNo < 0) alpha = Ng / dNo;
        }
        for (int i = 1; i < nc; ++i) {
          if (N.N[i] == 0) continue;
          const double dNo = alpha * x[i - 1];
          oil.N[i] += dNo;
          gas.N[i] += -dNo;
        }
        int e = op.calculate(c, t, p, T, oil);
        if (e) return e;
        e = gp.calculate(c, t, p, T, gas);
        if (e) return e;
      }
    } while ((res = residual(nc, op, gp)) > c.tol);
    return CUBIC_OK;
  }

  __device__ int molar_derivatives(const DCubic& c, const CComp& N, const CPhase& op, const CPhase& gp) {
    const int nc = c.nc, m = nc - 1, pi = nc - 1, Ti = pi + 1;
    double F[NCM * NCM], R[NCM * (NCM + 1)];
    int piv[NCM];
    for (int q = 0; q < m * m; ++q) F[q] = 0;
    for (int q = 0; q < m * (nc + 1); ++q) R[q] = 0;
    for (int i = 1; i < nc; ++i) {
      if (N.N[i] == 0) {
        F[(i - 1) + (i - 1) * m] = 1;
        continue;
      }
      R[(i - 1) + pi * m] = gp.dfdp[i] - op.dfdp[i];
      R[(i - 1) + Ti * m] = gp.dfdT[i] - op.dfdT[i];
      for (int j = 1; j < nc; ++j) {
        if (N.N[j] == 0) continue;
        F[(i - 1) + (j - 1) * m] = op.dfdN[i][j] + gp.dfdN[i][j];
        R[(i - 1) + (j - 1) * m] = gp.dfdN[i][j];
      }
    }
    if (small_lu(m, F, piv) > 0) return CUBIC_SINGULAR;
    for (int col = 0; col < nc + 1; ++col) small_solve(m, F, piv, R + col * m);
    for (int i = 1; i < nc; ++i) {
      dNodp[i] = R[(i - 1) + pi * m];
      dNodT[i] = R[(i - 1) + Ti * m];
      for (int j = 1; j < nc; ++j) dNodN[i][j] = R[(i - 1) + (j - 1) * m];
    }
    return CUBIC_OK;
  }
};

__device__ double lbc_viscosity(const DCubic& c, double T, const CComp& N, double xi) {
  const double c1 = 3.4e-4, c2 = 1.778e-4, c3 = 4.58, c4 = 1.67;
  const double e1 = 0.94, e2 = 0.625;
  const double Tdiv = 1.5;
  double Vcl = 0, Tcl = 0, Ml = 0, pcl = 0, M2l = 0, musl = 0;
  for (int i = 1; i < c.nc; ++i) {
    const double C = N.x(c.nc, i);
    const double M = c.Mw[i], Tc = c.Tc[i], pc = c.pc[i], Vc = c.Vc[i];
    Vcl += C * Vc;
    Tcl += C * Tc;
    Ml += C * M;
    pcl += C * pc;
    M2l += C * c.sqrtM[i];
    double mui = 0;
    const double Tr = T / Tc;
    if (Tr > Tdiv) mui = c1 * pow(Tr, e1);
    else mui = c2 * pow(c3 * Tr - c4, e2);
    mui *= c.zeta_inv[i];
    musl += C * mui * c.sqrtM[i];
  }
  musl /= M2l;
  const double zinv = sqrt(Ml) * pow(pcl, 2. / 3) / pow(Tcl, 1. / 6);
  const double xir = xi * Vcl;
  const double chi = c.lbc[0] + xir * (c.lbc[1] + xir * (c.lbc[2] + xir * (c.lbc[3] + xir * c.lbc[4])));
  const double mu = musl + zinv * (chi * chi * chi * chi - 1e-4);
  if (mu != mu) return 0;
  return mu * 1e-3;
}

// CubicEquationOfState.calculatePhaseState + WaterEquationOfState for one
// cell; ph = {water, oil, gas} in/out.  Returns a CUBIC_* code.
__device__ __noinline__ int cubic_phase_state(const DCubic& c, double p, double T, const double* Nin, Phase* ph, int* iters) {
  const int nc = c.nc;
  CComp N;
  for (int i = 0; i < NCM; ++i) N.N[i] = i < nc ? Nin[i] : 0;
  auto set_present = [&](Phase& d, bool exists) {
    d.present = exists;
    if (!exists) {
      d.V = d.xi = d.dVdp = d.dVdT = d.h = d.dhdT = d.mu = 0;
      for (int i = 0; i < nc; ++i) d.N[i] = d.dVdN[i] = 0;
    }
  };
  {
    Phase& w = ph[0];
    const double Nw = N.N[0];
    double pT[2] = {p, T};
    if (Nw > 0) {
      set_present(w, true);
      const double xiw = f_eval(c.wden, -1, pT);
      const double Vw = Nw / xiw;
      w.xi = xiw;
      w.V = Vw;
      w.N[0] = Nw;
      const double dxiw_dp = f_eval(c.wden, 0, pT);
      const double dxiw_dT = f_eval(c.wden, 1, pT);
      if (dxiw_dp < 0) return CUBIC_WATER;
      w.dVdp = -(Vw / xiw) * dxiw_dp;
      w.dVdT = -(Vw / xiw) * dxiw_dT;
      w.dVdN[0] = 1 / xiw;
      w.mu = f_eval(c.wvis, -1, pT);
    } else {
      set_present(w, false);
    }
  }
  CTemp t;
  cubic_update(c, T, t);
  CPhase op, gp;
  op.oil = true;
  gp.oil = false;
  CComp oil, gas;
  for (int i = 0; i < NCM; ++i) {
    oil.N[i] = i < nc ? ph[1].N[i] : 0;
    gas.N[i] = i < nc ? ph[2].N[i] : 0;
  }
  CFlash fl;
  const int e = fl.flash(c, t, p, T, N, oil, gas, op, gp);
  *iters = fl.iterations;
  if (e) return e;
  for (int i = 1; i < nc; ++i)
    if (N.N[i] == 0) {
      oil.N[i] = 0;
      gas.N[i] = 0;
    }
  Phase& od = ph[1];
  Phase& gd = ph[2];
  set_present(od, oil.NT(nc) > 0);
  set_present(gd, gas.NT(nc) > 0);
  if (od.present)
    for (int i = 0; i < nc; ++i) od.N[i] = oil.N[i];
  if (gd.present)
    for (int i = 0; i < nc; ++i) gd.N[i] = gas.N[i];
  const double RT = CUBIC_R * T;
  if (od.present) {
    od.V = op.Z * oil.NT(nc) * RT / p;
    od.xi = p / (op.Z * RT);
  }
  if (gd.present) {
    gd.V = gp.Z * gas.NT(nc) * RT / p;
    gd.xi = p / (gp.Z * RT);
  }
  auto single = [&](const CPhase& pp, Phase& d, const CComp& comp) {
    const double V = d.V, Z = pp.Z;
    d.dVdp = (V / Z) * pp.dZdp - V / p;
    d.dVdT = (V / Z) * pp.dZdT + V / T;
    const double Nl = comp.NT(nc);
    for (int i = 1; i < nc; ++i) d.dVdN[i] = (V / Z) * pp.dZdN[i] + V / Nl;
  };
  if (od.present && gd.present) {
    const int e2 = fl.molar_derivatives(c, N, op, gp);
    if (e2) return e2;
    const double Vo = od.V, Vg = gd.V, Zo = op.Z, Zg = gp.Z;
    double dZodp = op.dZdp, dZgdp = gp.dZdp, dZodT = op.dZdT, dZgdT = gp.dZdT;
    double dNodp = 0, dNodT = 0;
    for (int i = 1; i < nc; ++i) {
      dNodp += fl.dNodp[i];
      dNodT += fl.dNodT[i];
      dZodp += op.dZdN[i] * fl.dNodp[i];
      dZgdp -= gp.dZdN[i] * fl.dNodp[i];
      dZodT += op.dZdN[i] * fl.dNodT[i];
      dZgdT -= gp.dZdN[i] * fl.dNodT[i];
    }
    const double dNgdp = -dNodp, dNgdT = -dNodT;
    const double No = oil.NT(nc), Ng = gas.NT(nc);
    od.dVdp = (Vo / Zo) * dZodp + (Vo / No) * dNodp - Vo / p;
    gd.dVdp = (Vg / Zg) * dZgdp + (Vg / Ng) * dNgdp - Vg / p;
    od.dVdT = (Vo / Zo) * dZodT + (Vo / No) * dNodT + Vo / T;
    gd.dVdT = (Vg / Zg) * dZgdT + (Vg / Ng) * dNgdT + Vg / T;
    for (int i = 1; i < nc; ++i) {
      double dVodNi = 0, dVgdNi = 0;
      for (int j = 1; j < nc; ++j) {
        if (N.N[j] == 0) continue;
        const double dNodNi = fl.dNodN[j][i];
        double dNgdNi = -dNodNi;
        if (i == j) dNgdNi++;
        const double dZodN = op.dZdN[j], dZgdN = gp.dZdN[j];
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
  if (od.present) od.mu = lbc_viscosity(c, T, oil, od.xi);
  if (gd.present) gd.mu = lbc_viscosity(c, T, gas, gd.xi);
  return CUBIC_OK;
}

// One thread per cell over the rsg_cubic_phase_state layout.
__global__ void __launch_bounds__(128) k_cubic_phase_state(DCubic c, int n, const double* __restrict__ p,
                                                           const double* __restrict__ T,
                                                           const double* __restrict__ N, double* __restrict__ phases,
                                                           int* __restrict__ iters, int* __restrict__ err,
                                                           int* __restrict__ cell_status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nc = c.nc, nf = 6 + 2 * nc;
  double Ni[NCM];
  for (int nu = 0; nu < nc; ++nu) Ni[nu] = N[(int64_t)nu * n + i];
  Phase ph[3];
  for (int a = 0; a < 3; ++a) {
    auto at = [&](int f) { return phases[((int64_t)a * nf + f) * n + i]; };
    ph[a].present = at(0) != 0;
    ph[a].V = at(1);
    ph[a].xi = at(2);
    ph[a].dVdp = at(3);
    ph[a].dVdT = at(4);
    ph[a].mu = at(5);
    ph[a].h = ph[a].dhdT = 0;
    for (int nu = 0; nu < NCM; ++nu) {
      ph[a].N[nu] = nu < nc ? at(6 + nu) : 0;
      ph[a].dVdN[nu] = nu < nc ? at(6 + nc + nu) : 0;
    }
  }
  int it = 0;
  const int e = cubic_phase_state(c, p[i], T[i], Ni, ph, &it);
  iters[i] = it;
  if (e) atomicMin(err, e * (1 << 24) + i);
  if (cell_status) cell_status[i] = e == CUBIC_OK ? RSG_OK : (e == CUBIC_SINGULAR ? RSG_SINGULAR : RSG_PHYSICS);
  for (int a = 0; a < 3; ++a) {
    double* base = phases + (int64_t)a * nf * n + i;
    base[0] = ph[a].present ? 1 : 0;
    base[(int64_t)1 * n] = ph[a].V;
    base[(int64_t)2 * n] = ph[a].xi;
    base[(int64_t)3 * n] = ph[a].dVdp;
    base[(int64_t)4 * n] = ph[a].dVdT;
    base[(int64_t)5 * n] = ph[a].mu;
    for (int nu = 0; nu < nc; ++nu) {
      base[(int64_t)(6 + nu) * n] = ph[a].N[nu];
      base[(int64_t)(6 + nc + nu) * n] = ph[a].dVdN[nu];
    }
  }
}
