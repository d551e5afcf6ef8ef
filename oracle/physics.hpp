// Oracle (test infrastructure only): restatement of RS's per-cell property
// chain (CV), per-connection Darcy fluxes (CS), field initialisation and the
// sequential pressure/explicit-mass time step (Discretisation) for black-oil
// fluids with Corey relative permeabilities.
//
// Reference files (under rs/src/no/uib/cipr/rs/):
//   util/LookupTable.java:202-430, util/EvenLookupTable.java:81-175,
//   util/ConstantValue.java
//   fluid/WaterEquationOfState.java:71-129, fluid/BlackOilEquationOfState.java:168-547
//   fluid/EquationOfStateData.java:104-316, fluid/Composition.java:64-124
//   rock/CoreyRockFluid.java:84-141
//   field/CV.java:375-550, field/CS.java:94-170, field/Field.java:260-501
//   numerics/Discretisation.java:208-919, numerics/LinearSolver.java:244-302
#pragma once
#include <memory>
#include <vector>

#include "../include/rsg.h"
#include "mesh.hpp"
#include "mtj.hpp"

namespace orc {

// util/Function implementations
struct Function {
  int kind = RSG_FN_CONSTANT;
  int dim = 1;
  double value = 0;
  int n[3] = {1, 1, 1};
  std::vector<double> coord[3];
  double offset[3] = {0, 0, 0}, delta[3] = {0, 0, 0};
  std::vector<double> data;
  Function() {}
  explicit Function(const rsg_function& f);
  double get(const double* x) const { return evaluate(-1, x); }
  double deriv(int d, const double* x) const { return evaluate(d, x); }
  double evaluate(int n, const double* x) const;
  int getIndex(int d, double x) const;
  double getWeight(int d, int index, double x) const;
  double minOutput() const;
  double maxOutput() const;
};

enum { WATER = 0, OIL = 1, GAS = 2 };

struct EOSData {  // fluid/EquationOfStateData.java
  bool present = false;
  double V = 0, xi = 0, dVdp = 0, dVdT = 0, h = 0, dhdT = 0, mu = 0;
  double N[RSG_MAX_COMPONENTS] = {0};
  double dVdN[RSG_MAX_COMPONENTS] = {0};
  void setNotPresent(int nc);
  double NT(int nc) const;
};

struct BlackOil {
  int nc = 2;
  double Mw[RSG_MAX_COMPONENTS] = {0};
  std::vector<int> O, G;
  Function waterDensity, waterViscosity, waterEnthalpy, bubblePoint, dewPoint, oilDensity, gasDensity, oilViscosity,
      gasViscosity, oilEnthalpy, gasEnthalpy;
  explicit BlackOil(const rsg_blackoil& f);
  void calculatePhaseState(double p, const double* N, double T, EOSData* data) const;
};

// CoreyRockFluid, or (kind != RSG_RF_COREY) TabularRockFluid /
// ThreePhaseTabularRockFluid
struct Corey {
  rsg_corey c;
  int kind = RSG_RF_COREY;
  Function krw, krg, krow, krog, kro, pcowF, pcgoF;
  void setTables(const rsg_rock_tables& t);
  double effectiveSaturation(int phase, double S) const;
  void relperm(const double* S, double* kr) const;
  double pcow(const double* S) const;
  double pcgo(const double* S) const;
};

// field/CV.java state per control volume
struct CVState {
  double p = 0, p0 = 0, T = 0;
  double N[RSG_MAX_COMPONENTS] = {0};
  EOSData eos[3];
  double delta = 0, phi = 0, pcow = 0, pcgo = 0;
  double kr[3] = {0}, S[3] = {0}, rho[3] = {0}, lambda[3] = {0};
  double R = 0, dRdp = 0, dRdT = 0;
  double dRdN[RSG_MAX_COMPONENTS] = {0};
  double compMob[RSG_MAX_COMPONENTS][3] = {{0}};
  double phasePressure(int ph) const { return ph == WATER ? p - pcow : (ph == OIL ? p : p + pcgo); }
};

struct CSState {  // field/CS.java
  double u[3] = {0}, rho[3] = {0};
  int upstream[3] = {0};
};

struct Simulator {
  const Mesh* mesh;
  BlackOil eos;
  Corey rockFluid;
  int nc;
  std::vector<double> phi0, cr, heatCap;
  std::vector<CVState> cv;
  std::vector<CSState> cs;
  std::vector<rsg_source> sources;
  std::vector<std::vector<int>> sourceElements;
  rsg_runspec spec;
  double omega, ax, ay;
  std::vector<int> locked;
  CompRowMatrix A;      // LinearSolver.A
  std::unique_ptr<Preconditioner> M;
  Vec b, x;
  // state at the previous time step (Discretisation.p, T, R, N)
  std::vector<double> p_prev, T_prev, R_prev, N_prev;
  std::vector<double> dp;
  std::vector<double> dN;  // nc * n
  std::vector<double> dNfull;  // nc * n, the last step's dN before the locks
  // diagnostics of the last assembled system
  Vec lastJ, lastRhs;
  int lastLinearIterations = 0;
  double massBalance = 0;
  double time = 0, lastDt = 0;  // Field.t, the last attempted step
  int pressureIterations = 0;   // PressureNewtonRaphson.pressureIterations

  // compositional runs: the cubic equation of state replaces the black-oil one
  bool useCubic = false;
  rsg_cubic_fluid cubic{};
  Function cubicWden, cubicWvis;

  Simulator(const Mesh& mesh, const rsg_blackoil& fluid, const rsg_corey& rf, const double* poro, const double* comp,
            int nsources, const rsg_source* src, const rsg_initial& init, const rsg_runspec& spec,
            const rsg_cubic_fluid* cubicFluid = nullptr);

  double bodyForce(int el) const;
  void cvSecondaries(int i);
  void csSecondaries(int c);
  void calculateSecondaries();
  void volumeBalanceInit(const rsg_initial& init);
  void volumeBalance(const rsg_initial& init, const double* C, int el);

  // Discretisation.solve(dt); returns the Newton iteration count.
  int step(double dt, rsg_step_info* info);
  void storeCurrentState();
  void assembleFlux();
  void assembleDiagonal(double dt);
  int linearSolve();  // LinearSolver.solve
  double updatePressure();
  void molarMass(double dt);
  void retract();
  // Discretisation.calculateDt and its factors (:928-1002)
  double dtFactor(double value, double target, const rsg_dt_control& c) const;
  double residualVolumeFactor(const rsg_dt_control& c) const;
  double throughputFactor(const rsg_dt_control& c) const;
  double calculateDt(double dt, const rsg_dt_control& c, rsg_dt_factors* f) const;
  // TimeStepper.stepTo (numerics/TimeStepper.java:58-102)
  int stepTo(double endTime, const rsg_dt_control& c, double& dt, rsg_step_to_info* info);
};

// Cubic equation of state (cubic.cpp): CubicEquationOfState.calculatePhaseState
// for one cell; ph = {water, oil, gas} in/out; returns the flash iterations.
int cubic_phase_state(const rsg_cubic_fluid& fl, const Function& wden, const Function& wvis, double p, double T,
                      const double* N, EOSData* ph);
void cubic_roots_kat(double a0, double a1, double a2, double* z);  // CubicEquation roots, ascending

}  // namespace orc
