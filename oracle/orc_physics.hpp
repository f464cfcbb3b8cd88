// Oracle -- test infrastructure only (the checker, never the product).
// Pointwise physics restated from the reference:
//   variable conversion : src/Solver/VariableConvertor.cpp:315-421 (conserved/computational/primitive)
//   gradient conversion : src/Solver/VariableConvertor.cpp:574-620
//   convective fluxes   : src/Solver/ConvectiveFlux.cpp:27-350 (raw, normal, central, LF, HLLC, Roe)
//   viscous fluxes      : src/Solver/ViscousFlux.cpp:25-170
//   physical model      : src/Solver/PhysicalModel.cpp:26-165
//   boundary conditions : src/Solver/BoundaryCondition.cpp:79-547
//   incompressible model: PhysicalModel.cpp:57-78 (weakly compressible EOS), ConvectiveFlux.cpp:45-91,352-414
//                         (rho e flux, Exact flux), VariableConvertor.cpp:310-337,598-612, ViscousFlux.cpp:84-101,
//                         BoundaryCondition.cpp:153-180,243-270 (farfield star state), SourceTerm.cpp:29-58
#pragma once
#include <algorithm>
#include <cmath>

namespace orc {

constexpr int kMaxVar = 5;

struct Physics {
  int dim = 2;
  Real gamma = 1.4, cp = 0, cv = 0, mu = 0, pr = 0.71, kappa = 0;
  int transport = 1;  // 1 constant, 2 Sutherland
  // incompressible model: last conserved variable rho e, p = c0^2 (rho - rho0) + 0.01 rho0 c0^2, sound speed c0
  bool incomp = false;
  Real c0 = 0, rho0 = 0, padd = 0;
  // Boussinesq source rho beta (T - Tref) g on the last momentum component, g = 1
  int source = 0;
  Real beta = 0, tref = 0;
  Real temperatureFromInternalEnergy(Real e) const { return e / cv; }
  Real internalEnergyFromTemperature(Real t) const { return cv * t; }
  Real pressure(Real rho, Real e) const { return incomp ? c0 * c0 * (rho - rho0) + padd : (gamma - 1.0) * rho * e; }
  Real soundSpeed(Real rho, Real p) const { return incomp ? c0 : std::sqrt(gamma * p / rho); }
  Real entropy(Real rho, Real p) const { return p / std::pow(rho, gamma); }
  Real sutherlandRatio(Real t) const {
    const Real s = Real(110.4) / Real(273.15);
    return std::sqrt(t * t * t) * (1.0 + s) / (t + s);
  }
  Real viscosity(Real t) const { return transport == 2 ? mu * sutherlandRatio(t) : mu; }
  Real conductivity(Real t) const { return transport == 2 ? kappa * sutherlandRatio(t) : kappa; }
};

// Conserved (rho, m, rhoE) + computational (rho, u, e, p) of one point.
struct PointVar {
  Real cons[kMaxVar];
  Real rho, u[3], e, p;
  Real u2(int d) const { Real s = 0; for (int k = 0; k < d; ++k) s += u[k] * u[k]; return s; }
};

inline void computationalFromConserved(const Physics& ph, PointVar& v) {
  const int d = ph.dim;
  v.rho = v.cons[0];
  for (int k = 0; k < d; ++k) v.u[k] = v.cons[1 + k] / v.rho;
  v.e = ph.incomp ? v.cons[d + 1] / v.rho : v.cons[d + 1] / v.rho - v.u2(d) / 2.0;
  v.p = ph.pressure(v.rho, v.e);
}
inline void conservedFromComputational(const Physics& ph, PointVar& v) {
  const int d = ph.dim;
  v.cons[0] = v.rho;
  for (int k = 0; k < d; ++k) v.cons[1 + k] = v.rho * v.u[k];
  v.cons[d + 1] = ph.incomp ? v.rho * v.e : v.rho * (v.e + v.u2(d) / 2.0);
}
// primitive (rho, u, T) -> conserved and computational (VariableConvertor.cpp:341-380).
inline void fromPrimitive(const Physics& ph, const Real* prim, PointVar& v) {
  const int d = ph.dim;
  v.rho = prim[0];
  for (int k = 0; k < d; ++k) v.u[k] = prim[1 + k];
  v.e = ph.internalEnergyFromTemperature(prim[d + 1]);
  v.p = ph.pressure(v.rho, v.e);
  conservedFromComputational(ph, v);
}

// Normal convective flux F(U).n (ConvectiveFlux.cpp:59-91), from the computational variables.
inline void normalFlux(const Physics& ph, const Real* n, const PointVar& v, Real* f) {
  const int d = ph.dim;
  Real un = 0; for (int k = 0; k < d; ++k) un += v.u[k] * n[k];
  f[0] = v.rho * un;
  for (int k = 0; k < d; ++k) f[1 + k] = v.rho * un * v.u[k] + v.p * n[k];
  const Real et = v.e + v.u2(d) / 2.0;
  f[d + 1] = ph.incomp ? v.rho * v.e * un : (v.rho * et + v.p) * un;
}

// Raw convective flux F (d x nv, [k][var]) (ConvectiveFlux.cpp:27-57).
inline void rawFlux(const Physics& ph, const PointVar& v, Real f[3][kMaxVar]) {
  const int d = ph.dim;
  const Real et = v.e + v.u2(d) / 2.0;
  for (int k = 0; k < d; ++k) {
    f[k][0] = v.rho * v.u[k];
    for (int m = 0; m < d; ++m) f[k][1 + m] = v.rho * v.u[k] * v.u[m] + (k == m ? v.p : 0.0);
    f[k][d + 1] = ph.incomp ? v.rho * v.e * v.u[k] : (v.rho * et + v.p) * v.u[k];
  }
}

inline void centralFlux(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, Real* h) {
  Real fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  for (int i = 0; i < ph.dim + 2; ++i) h[i] = (fl[i] + fr[i]) / 2.0;
}

inline void laxFriedrichsFlux(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, Real* h) {
  const int d = ph.dim;
  Real fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  Real unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  const Real cl = ph.soundSpeed(l.rho, l.p), cr = ph.soundSpeed(r.rho, r.p);
  const Real sr = std::max<Real>(std::fabs(unl) + cl, std::fabs(unr) + cr);
  for (int i = 0; i < d + 2; ++i) h[i] = ((fl[i] + fr[i]) - sr * (r.cons[i] - l.cons[i])) / 2.0;
}

inline void hllcFlux(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, Real* h) {
  const int d = ph.dim;
  const Real g = ph.gamma;
  Real unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  const Real cl = ph.soundSpeed(l.rho, l.p), cr = ph.soundSpeed(r.rho, r.p);
  const Real rhoAvg = (l.rho + r.rho) / 2.0, cAvg = (cl + cr) / 2.0;
  const Real ps = std::max<Real>(0.0, (l.p + r.p) / 2.0 - (unr - unl) * rhoAvg * cAvg);
  const Real sl = unl - cl * (ps <= l.p ? 1.0 : std::sqrt(1.0 + (g + 1.0) * (ps / l.p - 1.0) / 2.0 / g));
  if (sl >= 0.0) { normalFlux(ph, n, l, h); return; }
  const Real sr = unr + cr * (ps <= r.p ? 1.0 : std::sqrt(1.0 + (g + 1.0) * (ps / r.p - 1.0) / 2.0 / g));
  if (sr <= 0.0) { normalFlux(ph, n, r, h); return; }
  const Real ss = (r.p - l.p + l.rho * unl * (sl - unl) - r.rho * unr * (sr - unr)) /
                    (l.rho * (sl - unl) - r.rho * (sr - unr));
  const PointVar& s = ss >= 0.0 ? l : r;
  const Real sk = ss >= 0.0 ? sl : sr;
  const Real un = ss >= 0.0 ? unl : unr;
  Real f[kMaxVar], star[kMaxVar];
  normalFlux(ph, n, s, f);
  star[0] = s.rho * (sk - un) / (sk - ss);
  for (int k = 0; k < d; ++k) star[1 + k] = ((sk - un) * s.rho * s.u[k] + (ps - s.p) * n[k]) / (sk - ss);
  star[d + 1] = ((sk - un) * s.rho * (s.e + s.u2(d) / 2.0) - s.p * un + ps * ss) / (sk - ss);
  for (int i = 0; i < d + 2; ++i) h[i] = f[i] + sk * (star[i] - s.cons[i]);
}

inline void roeFlux(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, Real* h) {
  const int d = ph.dim, nv = d + 2;
  const Real g = ph.gamma;
  Real fl[kMaxVar], fr[kMaxVar];
  normalFlux(ph, n, l, fl); normalFlux(ph, n, r, fr);
  const Real sl = std::sqrt(l.rho), sr = std::sqrt(r.rho), ssum = sl + sr;
  const Real rho = std::sqrt(l.rho * r.rho);
  Real u[3] = {0, 0, 0};
  for (int k = 0; k < d; ++k) u[k] = (sl * l.u[k] + sr * r.u[k]) / ssum;
  Real u2 = 0; for (int k = 0; k < d; ++k) u2 += u[k] * u[k];
  const Real hl = l.e * g + l.u2(d) / 2.0, hr = r.e * g + r.u2(d) / 2.0;
  const Real ht = (sl * hl + sr * hr) / ssum;
  const Real e = (ht - u2 / 2.0) / g;
  const Real p = ph.pressure(rho, e);
  Real un = 0; for (int k = 0; k < d; ++k) un += u[k] * n[k];
  const Real c = ph.soundSpeed(rho, p);
  const Real drho = r.rho - l.rho, dp = r.p - l.p;
  Real du[3] = {0, 0, 0}; Real dun = 0;
  for (int k = 0; k < d; ++k) { du[k] = r.u[k] - l.u[k]; dun += du[k] * n[k]; }
  const Real delta = c / 20.0;
  const Real a1 = std::fabs(un - c) > delta ? std::fabs(un - c) : ((un - c) * (un - c) + delta * delta) / (2.0 * delta);
  const Real a4 = std::fabs(un + c) > delta ? std::fabs(un + c) : ((un + c) * (un + c) + delta * delta) / (2.0 * delta);
  Real col[4][kMaxVar];
  {
    const Real s = a1 * (dp - rho * c * dun) / (2.0 * c * c);
    col[0][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[0][1 + k] = (u[k] - c * n[k]) * s;
    col[0][d + 1] = (ht - c * un) * s;
  }
  {
    const Real s = std::fabs(un) * (drho - dp / (c * c));
    col[1][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[1][1 + k] = u[k] * s;
    col[1][d + 1] = u2 / 2.0 * s;
  }
  {
    const Real s = std::fabs(un) * rho;
    Real udu = 0; for (int k = 0; k < d; ++k) udu += u[k] * du[k];
    col[2][0] = 0.0;
    for (int k = 0; k < d; ++k) col[2][1 + k] = (du[k] - dun * n[k]) * s;
    col[2][d + 1] = (udu - un * dun) * s;
  }
  {
    const Real s = a4 * (dp + rho * c * dun) / (2.0 * c * c);
    col[3][0] = 1.0 * s;
    for (int k = 0; k < d; ++k) col[3][1 + k] = (u[k] + c * n[k]) * s;
    col[3][d + 1] = (ht + c * un) * s;
  }
  for (int i = 0; i < nv; ++i) h[i] = ((fl[i] + fr[i]) - (col[0][i] + col[1][i] + col[2][i] + col[3][i])) / 2.0;
}

// Star state of the incompressible model between l and r across n (ConvectiveFlux.cpp:352-414; the
// farfield condition uses the same state, BoundaryCondition.cpp:153-180,243-270): rho* from the two densities
// and the normal-velocity jump, un* from their mean and the density ratio; e* and the tangential velocity come
// from the upwind side (r when un* < 0), with rho* e* = rho_k e_k.
inline void exactStarState(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, bool upwindRight,
                           PointVar& s) {
  const int d = ph.dim;
  const Real c = ph.c0;
  Real unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  s.rho = std::sqrt(l.rho * r.rho * std::exp((unl - unr) / c));
  const Real uns = (unl + unr) / 2.0 + std::log(l.rho / r.rho) * c / 2.0;
  const PointVar& k = upwindRight ? r : l;
  const Real unk = upwindRight ? unr : unl;
  s.e = k.e * k.rho / s.rho;
  for (int j = 0; j < 3; ++j) s.u[j] = 0.0;
  for (int j = 0; j < d; ++j) s.u[j] = k.u[j] + (uns - unk) * n[j];
  s.p = ph.pressure(s.rho, s.e);
}

inline void exactFlux(const Physics& ph, const Real* n, const PointVar& l, const PointVar& r, Real* h) {
  const int d = ph.dim;
  const Real c = ph.c0;
  Real unl = 0, unr = 0; for (int k = 0; k < d; ++k) { unl += l.u[k] * n[k]; unr += r.u[k] * n[k]; }
  const Real uns = (unl + unr) / 2.0 + std::log(l.rho / r.rho) * c / 2.0;
  PointVar s{};
  exactStarState(ph, n, l, r, uns < 0.0, s);
  normalFlux(ph, n, s, h);
}

inline void convectiveFlux(const Physics& ph, int kind, const Real* n, const PointVar& l, const PointVar& r,
                           Real* h) {
  switch (kind) {
    case 0: centralFlux(ph, n, l, r, h); break;
    case 1: laxFriedrichsFlux(ph, n, l, r, h); break;
    case 2: hllcFlux(ph, n, l, r, h); break;
    case 3: roeFlux(ph, n, l, r, h); break;
    default: exactFlux(ph, n, l, r, h); break;
  }
}

// Primitive gradients (rho, u, T) from conserved gradients (VariableConvertor.cpp:574-620).
// cg / pg layout: [var*d + dir].
inline void primitiveGradient(const Physics& ph, const PointVar& v, const Real* cg, Real* pg) {
  const int d = ph.dim;
  Real drho[3], gu[3][3];  // gu[j][m] = d_j u_m
  for (int j = 0; j < d; ++j) { drho[j] = cg[0 * d + j]; pg[0 * d + j] = drho[j]; }
  for (int m = 0; m < d; ++m)
    for (int j = 0; j < d; ++j) {
      gu[j][m] = (cg[(1 + m) * d + j] - drho[j] * v.u[m]) / v.rho;
      pg[(1 + m) * d + j] = gu[j][m];
    }
  const Real et = v.cons[d + 1] / v.rho;  // total (compressible) or internal (incompressible) energy per mass
  for (int j = 0; j < d; ++j) {
    Real ge = (cg[(d + 1) * d + j] - drho[j] * et) / v.rho;
    if (!ph.incomp)
      for (int m = 0; m < d; ++m) ge -= gu[j][m] * v.u[m];
    pg[(d + 1) * d + j] = ph.temperatureFromInternalEnergy(ge);
  }
}

// Viscous normal flux F_v(U, grad).n (ViscousFlux.cpp:58-103,115-127); pg = primitive gradient.
inline void viscousNormalFlux(const Physics& ph, const Real* n, const PointVar& v, const Real* pg, Real* f) {
  const int d = ph.dim;
  Real gu[3][3];
  for (int j = 0; j < d; ++j)
    for (int m = 0; m < d; ++m) gu[j][m] = pg[(1 + m) * d + j];
  const Real t = ph.temperatureFromInternalEnergy(v.e);
  const Real mu = ph.viscosity(t);
  Real tr = 0; for (int j = 0; j < d; ++j) tr += gu[j][j];
  Real tau[3][3];
  for (int j = 0; j < d; ++j)
    for (int m = 0; m < d; ++m) tau[j][m] = mu * (gu[j][m] + gu[m][j]) - (j == m ? 2.0 / 3.0 * mu * tr : 0.0);
  const Real kap = ph.conductivity(t);
  Real raw[3][kMaxVar];
  for (int k = 0; k < d; ++k) {
    raw[k][0] = 0.0;
    for (int m = 0; m < d; ++m) raw[k][1 + m] = tau[k][m];
    Real tu = 0;
    if (!ph.incomp) for (int m = 0; m < d; ++m) tu += tau[k][m] * v.u[m];  // incompressible: conduction only
    raw[k][d + 1] = tu + kap * pg[(d + 1) * d + k];
  }
  for (int i = 0; i < d + 2; ++i) { Real s = 0; for (int k = 0; k < d; ++k) s += raw[k][i] * n[k]; f[i] = s; }
}

// ---- boundary conditions (BoundaryCondition.cpp:79-547) -------------------------------------------
// ghost: boundary dummy state (user primitive at the face point); out: boundary state (computational).
inline void boundaryState(const Physics& ph, int bc, const Real* n, const PointVar& l, const PointVar& ghost,
                          PointVar& b) {
  const int d = ph.dim;
  const Real g = ph.gamma;
  Real unl = 0; for (int k = 0; k < d; ++k) unl += l.u[k] * n[k];
  const Real mn = unl / ph.soundSpeed(l.rho, l.p);
  auto copyComp = [&](const PointVar& s) { b.rho = s.rho; for (int k = 0; k < 3; ++k) b.u[k] = s.u[k]; b.e = s.e; b.p = s.p; };
  switch (bc) {
    case 0: {  // RiemannFarfield
      if (std::fabs(mn) > 1.0) { copyComp(mn < 0.0 ? ghost : l); break; }
      if (ph.incomp) {  // the exact-flux star state, internal energy and tangential velocity from the upwind side
        exactStarState(ph, n, l, ghost, mn < 0.0, b);
        break;
      }
      Real ung = 0; for (int k = 0; k < d; ++k) ung += ghost.u[k] * n[k];
      const Real rm = ung - 2.0 * ph.soundSpeed(ghost.rho, ghost.p) / (g - 1.0);
      const Real rp = unl + 2.0 * ph.soundSpeed(l.rho, l.p) / (g - 1.0);
      const Real unb = (rm + rp) / 2.0;
      const PointVar& side = mn < 0.0 ? ghost : l;
      Real uns = 0; for (int k = 0; k < d; ++k) uns += side.u[k] * n[k];
      for (int k = 0; k < d; ++k) b.u[k] = side.u[k] + (unb - uns) * n[k];
      const Real cb = (g - 1.0) * (rp - rm) / 4.0;
      const Real sb = ph.entropy(side.rho, side.p);
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
inline void boundaryGradientState(const Physics& ph, int bc, const Real* n, const PointVar& l, const PointVar& ghost,
                                  Real* volume, Real* interface) {
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
