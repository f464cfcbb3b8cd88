// Oracle -- test infrastructure only (the checker, never the product).
// Pointwise physics restated from the reference:
//   variable conversion : src/Solver/VariableConvertor.cpp:315-421 (conserved/computational/primitive)
//   gradient conversion : src/Solver/VariableConvertor.cpp:574-620
//   convective fluxes   : src/Solver/ConvectiveFlux.cpp:27-350 (raw, normal, central, LF, HLLC, Roe)
//   viscous fluxes      : src/Solver/ViscousFlux.cpp:25-170
//   physical model      : src/Solver/PhysicalModel.cpp:26-165
//   boundary conditions : src/Solver/BoundaryCondition.cpp:79-547
#pragma once
#include <algorithm>
#include <cmath>

namespace orc {

constexpr int kMaxVar = 5;

struct Physics {
  int dim = 2;
  double gamma = 1.4, cp = 0, cv = 0, mu = 0, pr = 0.71, kappa = 0;
  int transport = 1;  // 1 constant, 2 Sutherland
  double temperatureFromInternalEnergy(double e) const { return e / cv; }
  double internalEnergyFromTemperature(double t) const { return cv * t; }
  double pressure(double rho, double e) const { return (gamma - 1.0) * rho * e; }
  double soundSpeed(double rho, double p) const { return std::sqrt(gamma * p / rho); }
  double entropy(double rho, double p) const { return p / std::pow(rho, gamma); }
  double sutherlandRatio(double t) const {
    constexpr double s = 110.4 / 273.15;
    return std::sqrt(t * t * t) * (1.0 + s) / (t + s);
  }
  double viscosity(double t) const { return transport == 2 ? mu * sutherlandRatio(t) : mu; }
  double conductivity(double t) const { return transport == 2 ? kappa * sutherlandRatio(t) : kappa; }
};

// Conserved (rho, m, rhoE) + computational (rho, u, e, p) of one point.
struct PointVar {
  double cons[kMaxVar];
  double rho, u[3], e, p;
  double u2(int d) const { double s = 0; for (int k = 0; k < d; ++k) s += u[k] * u[k]; return s; }
};

inline void computationalFromConserved(const Physics& ph, PointVar& v) {
  const int d = ph.dim;
  v.rho = v.cons[0];
  for (int k = 0; k < d; ++k) v.u[k] = v.cons[1 + k] / v.rho;
  v.e = v.cons[d + 1] / v.rho - v.u2(d) / 2.0;
  v.p = ph.pressure(v.rho, v.e);
}
inline void conservedFromComputational(const Physics& ph, PointVar& v) {
  const int d = ph.dim;
  v.cons[0] = v.rho;
  for (int k = 0; k < d; ++k) v.cons[1 + k] = v.rho * v.u[k];
  v.cons[d + 1] = v.rho * (v.e + v.u2(d) / 2.0);
}
// primitive (rho, u, T) -> conserved and computational (VariableConvertor.cpp:341-380).
inline void fromPrimitive(const Physics& ph, const double* prim, PointVar& v) {
  const int d = ph.dim;
  v.rho = prim[0];
  for (int k = 0; k < d; ++k) v.u[k] = prim[1 + k];
  v.e = ph.internalEnergyFromTemperature(prim[d + 1]);
  v.p = ph.pressure(v.rho, v.e);
  conservedFromComputational(ph, v);
}

// Normal convective flux F(U).n (ConvectiveFlux.cpp:59-91), from the computational variables.
inline void normalFlux(const Physics& ph, const double* n, const PointVar& v, double* f) {
  const int d = ph.dim;
  double un = 0; for (int k = 0; k < d; ++k) un += v.u[k] * n[k];
  f[0] = v.rho * un;
  for (int k = 0; k < d; ++k) f[1 + k] = v.rho * un * v.u[k] + v.p * n[k];
  const double et = v.e + v.u2(d) / 2.0;
  f[d + 1] = (v.rho * et + v.p) * un;
}

// Raw convective flux F (d x nv, [k][var]) (ConvectiveFlux.cpp:27-57).
inline void rawFlux(const Physics& ph, const PointVar& v, double f[3][kMaxVar]) {
  const int d = ph.dim;
  const double et = v.e + v.u2(d) / 2.0;
  for (int k = 0; k < d; ++k) {
    f[k][0] = v.rho * v.u[k];
    for (int m = 0; m < d; ++m) f[k][1 + m] = v.rho * v.u[k] * v.u[m] + (k == m ? v.p : 0.0);
    f[k][d + 1] = (v.rho * et + v.p) * v.u[k];
  }
}

inline void centralFlux(const Physics& ph, const double* n, const PointVar& l, const PointVar& r, double* h) {
  double fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  for (int i = 0; i < ph.dim + 2; ++i) h[i] = (fl[i] + fr[i]) / 2.0;
}

inline void laxFriedrichsFlux(const Physics& ph, const double* n, const PointVar& l, const PointVar& r, double* h) {
  const int d = ph.dim;
  double fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  double unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  const double cl = ph.soundSpeed(l.rho, l.p), cr = ph.soundSpeed(r.rho, r.p);
  const double sr = std::max(std::fabs(unl) + cl, std::fabs(unr) + cr);
  for (int i = 0; i < d + 2; ++i) h[i] = ((fl[i] + fr[i]) - sr * (r.cons[i] - l.cons[i])) / 2.0;
}

inline void hllcFlux(const Physics& ph, const double* n, const PointVar& l, const PointVar& r, double* h) {
  const int d = ph.dim;
  const double g = ph.gamma;
  double unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  const double cl = ph.soundSpeed(l.rho, l.p), cr = ph.soundSpeed(r.rho, r.p);
  const double rhoAvg = (l.rho + r.rho) / 2.0, cAvg = (cl + cr) / 2.0;
  const double ps = std::max(0.0, (l.p + r.p) / 2.0 - (unr - unl) * rhoAvg * cAvg);
  const double sl = unl - cl * (ps <= l.p ? 1.0 : std::sqrt(1.0 + (g + 1.0) * (ps / l.p - 1.0) / 2.0 / g));
  if (sl >= 0.0) { normalFlux(ph, n, l, h); return; }
  const double sr = unr + cr * (ps <= r.p ? 1.0 : std::sqrt(1.0 + (g + 1.0) * (ps / r.p - 1.0) / 2.0 / g));
  if (sr <= 0.0) { normalFlux(ph, n, r, h); return; }
  const double ss = (r.p - l.p + l.rho * unl * (sl - unl) - r.rho * unr * (sr - unr)) /
                    (l.rho * (sl - unl) - r.rho * (sr - unr));
  const PointVar& s = ss >= 0.0 ? l : r;
  const double sk = ss >= 0.0 ? sl : sr;
  const double un = ss >= 0.0 ? unl : unr;
  double f[kMaxVar], star[kMaxVar];
  normalFlux(ph, n, s, f);
  star[0] = s.rho * (sk - un) / (sk - ss);
  for (int k = 0; k < d; ++k) star[1 + k] = ((sk - un) * s.rho * s.u[k] + (ps - s.p) * n[k]) / (sk - ss);
  star[d + 1] = ((sk - un) * s.rho * (s.e + s.u2(d) / 2.0) - s.p * un + ps * ss) / (sk - ss);
  for (int i = 0; i < d + 2; ++i) h[i] = f[i] + sk * (star[i] - s.cons[i]);
}

inline void roeFlux(const Physics& ph, const double* n, const PointVar& l, const PointVar& r, double* h) {
  const int d = ph.dim, nv = d + 2;
  const double g = ph.gamma;
  double fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  const double sl = std::sqrt(l.rho), sr = std::sqrt(r.rho), ssum = sl + sr;
  const double rho = std::sqrt(l.rho * r.rho);
  double u[3] = {0, 0, 0};
  for (int k = 0; k < d; ++k) u[k] = (sl * l.u[k] + sr * r.u[k]) / ssum;
  double u2 = 0; for (int k = 0; k < d; ++k) u2 += u[k] * u[k];
  const double hl = l.e * g + l.u2(d) / 2.0, hr = r.e * g + r.u2(d) / 2.0;
  const double ht = (sl * hl + sr * hr) / ssum;
  const double e = (ht - u2 / 2.0) / g;
  const double p = ph.pressure(rho, e);
  double un = 0; for (int k = 0; k < d; ++k) un += u[k] * n[k];
  const double c = ph.soundSpeed(rho, p);
  const double drho = r.rho - l.rho, dp = r.p - l.p;
  double du[3] = {0, 0, 0}; double dun = 0;
  for (int k = 0; k < d; ++k) { du[k] = r.u[k] - l.u[k]; dun += du[k] * n[k]; }
  const double delta = c / 20.0;
  const double a1 = std::fabs(un - c) > delta ? std::fabs(un - c) : ((un - c) * (un - c) + delta * delta) / (2.0 * delta);
  const double a4 = std::fabs(un + c) > delta ? std::fabs(un + c) : ((un + c) * (un + c) + delta * delta) / (2.0 * delta);
  double col[4][kMaxVar];
  {
    const double s = a1 * (dp - rho * c * dun) / (2.0 * c * c);
    col[0][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[0][1 + k] = (u[k] - c * n[k]) * s;
    col[0][d + 1] = (ht - c * un) * s;
  }
  {
    const double s = std::fabs(un) * (drho - dp / (c * c));
    col[1][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[1][1 + k] = u[k] * s;
    col[1][d + 1] = u2 / 2.0 * s;
  }
  {
    const double s = std::fabs(un) * rho;
    double udu = 0; for (int k = 0; k < d; ++k) udu += u[k] * du[k];
    col[2][0] = 0.0;
    for (int k = 0; k < d; ++k) col[2][1 + k] = (du[k] - dun * n[k]) * s;
    col[2][d + 1] = (udu - un * dun) * s;
  }
  {
    const double s = a4 * (dp + rho * c * dun) / (2.0 * c * c);
    col[3][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[3][1 + k] = (u[k] + c * n[k]) * s;
    col[3][d + 1] = (ht + c * un) * s;
  }
  for (int i = 0; i < nv; ++i) h[i] = ((fl[i] + fr[i]) - (col[0][i] + col[1][i] + col[2][i] + col[3][i])) / 2.0;
}

inline void convectiveFlux(const Physics& ph, int kind, const double* n, const PointVar& l, const PointVar& r,
                           double* h) {
  switch (kind) {
    case 0: centralFlux(ph, n, l, r, h); break;
    case 1: laxFriedrichsFlux(ph, n, l, r, h); break;
    case 2: hllcFlux(ph, n, l, r, h); break;
    default: roeFlux(ph, n, l, r, h); break;
  }
}

// Primitive gradients (rho, u, T) from conserved gradients (VariableConvertor.cpp:574-620).
// cg / pg layout: [var*d + dir].
inline void primitiveGradient(const Physics& ph, const PointVar& v, const double* cg, double* pg) {
  const int d = ph.dim;
  double drho[3], gu[3][3];  // gu[j][m] = d_j u_m
  for (int j = 0; j < d; ++j) { drho[j] = cg[0 * d + j]; pg[0 * d + j] = drho[j]; }
  for (int m = 0; m < d; ++m)
    for (int j = 0; j < d; ++j) {
      gu[j][m] = (cg[(1 + m) * d + j] - drho[j] * v.u[m]) / v.rho;
      pg[(1 + m) * d + j] = gu[j][m];
    }
  const double et = v.cons[d + 1] / v.rho;
  for (int j = 0; j < d; ++j) {
    double ge = (cg[(d + 1) * d + j] - drho[j] * et) / v.rho;
    for (int m = 0; m < d; ++m) ge -= gu[j][m] * v.u[m];
    pg[(d + 1) * d + j] = ph.temperatureFromInternalEnergy(ge);
  }
}

// Viscous normal flux F_v(U, grad).n (ViscousFlux.cpp:58-103,115-127); pg = primitive gradient.
inline void viscousNormalFlux(const Physics& ph, const double* n, const PointVar& v, const double* pg, double* f) {
  const int d = ph.dim;
  double gu[3][3];
  for (int j = 0; j < d; ++j)
    for (int m = 0; m < d; ++m) gu[j][m] = pg[(1 + m) * d + j];
  const double t = ph.temperatureFromInternalEnergy(v.e);
  const double mu = ph.viscosity(t);
  double tr = 0; for (int j = 0; j < d; ++j) tr += gu[j][j];
  double tau[3][3];
  for (int j = 0; j < d; ++j)
    for (int m = 0; m < d; ++m) tau[j][m] = mu * (gu[j][m] + gu[m][j]) - (j == m ? 2.0 / 3.0 * mu * tr : 0.0);
  const double kap = ph.conductivity(t);
  double raw[3][kMaxVar];
  for (int k = 0; k < d; ++k) {
    raw[k][0] = 0.0;
    for (int m = 0; m < d; ++m) raw[k][1 + m] = tau[k][m];
    double tu = 0; for (int m = 0; m < d; ++m) tu += tau[k][m] * v.u[m];
    raw[k][d + 1] = tu + kap * pg[(d + 1) * d + k];
  }
  for (int i = 0; i < d + 2; ++i) { double s = 0; for (int k = 0; k < d; ++k) s += raw[k][i] * n[k]; f[i] = s; }
}

// ---- boundary conditions (BoundaryCondition.cpp:79-547) -------------------------------------------
// ghost: boundary dummy state (user primitive at the face point); out: boundary state (computational).
inline void boundaryState(const Physics& ph, int bc, const double* n, const PointVar& l, const PointVar& ghost,
                          PointVar& b) {
  const int d = ph.dim;
  const double g = ph.gamma;
  double unl = 0; for (int k = 0; k < d; ++k) unl += l.u[k] * n[k];
  const double mn = unl / ph.soundSpeed(l.rho, l.p);
  auto copyComp = [&](const PointVar& s) { b.rho = s.rho; for (int k = 0; k < 3; ++k) b.u[k] = s.u[k]; b.e = s.e; b.p = s.p; };
  switch (bc) {
    case 0: {  // RiemannFarfield
      if (std::fabs(mn) > 1.0) { copyComp(mn < 0.0 ? ghost : l); break; }
      double ung = 0; for (int k = 0; k < d; ++k) ung += ghost.u[k] * n[k];
      const double rm = ung - 2.0 * ph.soundSpeed(ghost.rho, ghost.p) / (g - 1.0);
      const double rp = unl + 2.0 * ph.soundSpeed(l.rho, l.p) / (g - 1.0);
      const double unb = (rm + rp) / 2.0;
      const PointVar& side = mn < 0.0 ? ghost : l;
      double uns = 0; for (int k = 0; k < d; ++k) uns += side.u[k] * n[k];
      for (int k = 0; k < d; ++k) b.u[k] = side.u[k] + (unb - uns) * n[k];
      const double cb = (g - 1.0) * (rp - rm) / 4.0;
      const double sb = ph.entropy(side.rho, side.p);
      b.rho = std::pow(cb * cb / (g * sb), 1.0 / (g - 1.0));
      b.p = b.rho * cb * cb / g;
      b.e = b.p / ((g - 1.0) * b.rho);
      break;
    }
    case 1: {  // VelocityInflow
      copyComp(ghost);
      if (mn > -1.0) b.p = l.p;
      break;
    }
    case 2: {  // PressureOutflow
      copyComp(l);
      if (mn < 1.0) b.p = ghost.p;
      break;
    }
    case 3: {  // IsoThermalNonSlipWall
      b.rho = l.rho;
      for (int k = 0; k < d; ++k) b.u[k] = ghost.u[k];
      b.e = ghost.e;
      b.p = ph.pressure(b.rho, ghost.e);
      break;
    }
    case 4: {  // AdiabaticSlipWall
      copyComp(l);
      for (int k = 0; k < d; ++k) b.u[k] = l.u[k] - unl * n[k];
      break;
    }
    default: {  // AdiabaticNonSlipWall
      copyComp(l);
      for (int k = 0; k < d; ++k) b.u[k] = ghost.u[k];
      break;
    }
  }
}

// Gradient ghost values: volume-gradient state and interface-gradient jump (conserved).
inline void boundaryGradientState(const Physics& ph, int bc, const double* n, const PointVar& l, const PointVar& ghost,
                                  double* volume, double* interface) {
  const int nv = ph.dim + 2;
  if (bc <= 2) {
    for (int i = 0; i < nv; ++i) { volume[i] = l.cons[i]; interface[i] = 0.0; }
    return;
  }
  PointVar b{};
  boundaryState(ph, bc, n, l, ghost, b);
  conservedFromComputational(ph, b);
  for (int i = 0; i < nv; ++i) { volume[i] = b.cons[i]; interface[i] = b.cons[i] - l.cons[i]; }
}

}  // namespace orc
