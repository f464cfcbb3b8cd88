// Device-side pointwise physics of the GB300 DG path (FP64).
//
// Restates, for the GPU, the pointwise functions of the reference:
//   conserved -> computational      src/Solver/VariableConvertor.cpp:315-339
//   normal / raw convective flux    src/Solver/ConvectiveFlux.cpp:27-91
//   Central, Lax-Friedrichs, HLLC, Roe (Harten fix delta = c/20)   ConvectiveFlux.cpp:93-350
//   primitive gradients             src/Solver/VariableConvertor.cpp:574-620
//   viscous flux                    src/Solver/ViscousFlux.cpp:58-170
//   boundary ghost states           src/Solver/BoundaryCondition.cpp:79-547
// The arithmetic is reorganised to cut FP64 instructions (the GB300 FP64 pipe issues ~2 DFMA/clk/SM):
// one reciprocal of rho per point instead of d+1 divisions, and divisions as a hardware reciprocal
// estimate refined by Newton-Raphson.  Results agree with the reference formulas to round-off.
#pragma once
#include <cstdint>

namespace sdg {

struct Phys {
  double gamma, gm1, cv, inv_cv, cp, mu, kappa;
  int transport;  // 1 constant, 2 Sutherland
  double hllc_g2;  // (gamma + 1) / (2 gamma), the HLLC wave-speed factor
};

// Reciprocal: rcp.approx.ftz.f64 estimate refined by two Newton-Raphson steps r <- r + r(1 - x r)
// (the classical iteration for 1/x, e.g. P. Markstein, IBM J. Res. Dev. 34(1), 1990).  Each step at
// least doubles the number of correct bits; the result is within a few ulp of 1/x.
__device__ __forceinline__ double rcp(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  return r;
}

template <int D>
struct State {
  double r, m[D], E;   // conserved
  double ir, u[D], p;  // 1/rho, velocity, pressure
};

template <int D>
__device__ __forceinline__ void makeState(State<D>& s, const double* U, const Phys& ph) {
  s.r = U[0];
#pragma unroll
  for (int k = 0; k < D; ++k) s.m[k] = U[1 + k];
  s.E = U[D + 1];
  s.ir = rcp(s.r);
  double mu = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { s.u[k] = s.m[k] * s.ir; mu = fma(s.m[k], s.u[k], mu); }
  s.p = ph.gm1 * fma(-0.5, mu, s.E);
}

template <int D>
__device__ __forceinline__ double dotn(const double* a, const double* n) {
  double s = a[0] * n[0];
#pragma unroll
  for (int k = 1; k < D; ++k) s = fma(a[k], n[k], s);
  return s;
}

template <int D>
__device__ __forceinline__ void normalFlux(const State<D>& s, const double* n, double un, double* f) {
  f[0] = s.r * un;
#pragma unroll
  for (int k = 0; k < D; ++k) f[1 + k] = fma(s.m[k], un, s.p * n[k]);
  f[D + 1] = (s.E + s.p) * un;
}

template <int D>
__device__ __forceinline__ void fluxCentral(const State<D>& l, const State<D>& r, const double* n, double* h) {
  double fl[D + 2], fr[D + 2];
  normalFlux(l, n, dotn<D>(l.u, n), fl);
  normalFlux(r, n, dotn<D>(r.u, n), fr);
#pragma unroll
  for (int i = 0; i < D + 2; ++i) h[i] = 0.5 * (fl[i] + fr[i]);
}

template <int D>
__device__ __forceinline__ void fluxLaxFriedrichs(const State<D>& l, const State<D>& r, const double* n,
                                                  const Phys& ph, double* h) {
  const double unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  double fl[D + 2], fr[D + 2];
  normalFlux(l, n, unl, fl);
  normalFlux(r, n, unr, fr);
  const double cl = sqrt(ph.gamma * l.p * l.ir), cr = sqrt(ph.gamma * r.p * r.ir);
  const double sr = fmax(fabs(unl) + cl, fabs(unr) + cr);
  h[0] = 0.5 * fma(-sr, r.r - l.r, fl[0] + fr[0]);
#pragma unroll
  for (int k = 0; k < D; ++k) h[1 + k] = 0.5 * fma(-sr, r.m[k] - l.m[k], fl[1 + k] + fr[1 + k]);
  h[D + 1] = 0.5 * fma(-sr, r.E - l.E, fl[D + 1] + fr[D + 1]);
}

// HLLC with PVRS pressure estimate and Toro's wave-speed factors (ConvectiveFlux.cpp:136-238).
template <int D>
__device__ __forceinline__ void fluxHLLC(const State<D>& l, const State<D>& r, const double* n, const Phys& ph,
                                         double* h) {
  const double unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  const double cl = sqrt(ph.gamma * l.p * l.ir), cr = sqrt(ph.gamma * r.p * r.ir);
  const double rhoAvg = 0.5 * (l.r + r.r), cAvg = 0.5 * (cl + cr);
  const double ps = fmax(0.0, fma(-(unr - unl), rhoAvg * cAvg, 0.5 * (l.p + r.p)));
  const double g2 = ph.hllc_g2;
  const double ql = ps <= l.p ? 1.0 : sqrt(fma(g2, fma(ps, rcp(l.p), -1.0), 1.0));
  const double sl = fma(-cl, ql, unl);
  if (sl >= 0.0) { normalFlux(l, n, unl, h); return; }
  const double qr = ps <= r.p ? 1.0 : sqrt(fma(g2, fma(ps, rcp(r.p), -1.0), 1.0));
  const double sr = fma(cr, qr, unr);
  if (sr <= 0.0) { normalFlux(r, n, unr, h); return; }
  const double al = l.r * (sl - unl), ar = r.r * (sr - unr);
  const double ss = (r.p - l.p + al * unl - ar * unr) * rcp(al - ar);
  const bool left = ss >= 0.0;
  const State<D>& s = left ? l : r;
  const double sk = left ? sl : sr, un = left ? unl : unr, a = left ? al : ar;
  double f[D + 2];
  normalFlux(s, n, un, f);
  const double inv = rcp(sk - ss);
  // star state minus the side's conserved state, times the wave speed
  const double rs = a * inv;
  h[0] = fma(sk, rs - s.r, f[0]);
  const double dp = ps - s.p;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double ms = fma(a, s.u[k], dp * n[k]) * inv;
    h[1 + k] = fma(sk, ms - s.m[k], f[1 + k]);
  }
  const double Es = fma(a, s.E * s.ir, fma(ps, ss, -s.p * un)) * inv;
  h[D + 1] = fma(sk, Es - s.E, f[D + 1]);
}

// Roe flux with Harten's entropy fix, delta = c/20 (ConvectiveFlux.cpp:240-350).
template <int D>
__device__ __forceinline__ void fluxRoe(const State<D>& l, const State<D>& r, const double* n, const Phys& ph,
                                        double* h) {
  const double g = ph.gamma;
  const double unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  double fl[D + 2], fr[D + 2];
  normalFlux(l, n, unl, fl);
  normalFlux(r, n, unr, fr);
  const double sl = sqrt(l.r), sr = sqrt(r.r);
  const double is = rcp(sl + sr);
  const double wl = sl * is, wr = sr * is;
  const double rho = sl * sr;
  double u[D], u2 = 0.0, un = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { u[k] = fma(wl, l.u[k], wr * r.u[k]); u2 = fma(u[k], u[k], u2); un = fma(u[k], n[k], un); }
  // total enthalpy H = (E + p)/rho
  const double hl = (l.E + l.p) * l.ir, hr = (r.E + r.p) * r.ir;
  const double ht = fma(wl, hl, wr * hr);
  // c^2 = gamma p / rho with p = (gamma-1) rho e and e = (H - u^2/2)/gamma
  const double c2 = (g - 1.0) * fma(-0.5, u2, ht);
  const double c = sqrt(c2);
  const double ic2 = rcp(c2);
  const double drho = r.r - l.r, dp = r.p - l.p;
  double du[D], dun = 0.0, udu = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { du[k] = r.u[k] - l.u[k]; dun = fma(du[k], n[k], dun); udu = fma(u[k], du[k], udu); }
  const double delta = c * 0.05;
  const double lm = un - c, lp = un + c;
  const double a1 = fabs(lm) > delta ? fabs(lm) : fma(lm, lm, delta * delta) * (10.0 * rcp(c));
  const double a4 = fabs(lp) > delta ? fabs(lp) : fma(lp, lp, delta * delta) * (10.0 * rcp(c));
  const double aun = fabs(un);
  const double rc = rho * c;
  const double s1 = a1 * fma(-rc, dun, dp) * (0.5 * ic2);
  const double s2 = aun * fma(-dp, ic2, drho);
  const double s3 = aun * rho;
  const double s4 = a4 * fma(rc, dun, dp) * (0.5 * ic2);
  const double s14 = s1 + s4, d14 = (s4 - s1) * c;
  h[0] = 0.5 * (fl[0] + fr[0] - (s14 + s2));
#pragma unroll
  for (int k = 0; k < D; ++k)
    h[1 + k] = 0.5 * (fl[1 + k] + fr[1 + k] - fma(u[k], s14 + s2, fma(d14, n[k], s3 * fma(-dun, n[k], du[k]))));
  h[D + 1] = 0.5 * (fl[D + 1] + fr[D + 1] - fma(ht, s14, fma(d14, un, fma(0.5 * u2, s2, s3 * fma(-un, dun, udu)))));
}

template <int D, int FLUX>
__device__ __forceinline__ void convectiveFlux(const State<D>& l, const State<D>& r, const double* n, const Phys& ph,
                                               double* h) {
  if constexpr (FLUX == 0) fluxCentral<D>(l, r, n, h);
  else if constexpr (FLUX == 1) fluxLaxFriedrichs<D>(l, r, n, ph, h);
  else if constexpr (FLUX == 2) fluxHLLC<D>(l, r, n, ph, h);
  else fluxRoe<D>(l, r, n, ph, h);
}

// Computational variables (rho, u, e, p) used by the boundary states.
template <int D>
struct Comp {
  double r, u[D], e, p;
};

template <int D>
__device__ __forceinline__ void compFromState(const State<D>& s, Comp<D>& c) {
  c.r = s.r;
#pragma unroll
  for (int k = 0; k < D; ++k) c.u[k] = s.u[k];
  c.p = s.p;
  double u2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fma(s.u[k], s.u[k], u2);
  c.e = fma(-0.5, u2, s.E * s.ir);
}

template <int D>
__device__ __forceinline__ void normalFluxComp(const Comp<D>& c, const double* n, double* f) {
  const double un = dotn<D>(c.u, n);
  double u2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fma(c.u[k], c.u[k], u2);
  f[0] = c.r * un;
#pragma unroll
  for (int k = 0; k < D; ++k) f[1 + k] = fma(c.r * un, c.u[k], c.p * n[k]);
  f[D + 1] = fma(c.r, fma(0.5, u2, c.e), c.p) * un;
}

// Boundary state (BoundaryCondition.cpp:79-547): l = interior trace, g = ghost (user) state.
template <int D>
__device__ __forceinline__ void boundaryState(int bc, const double* n, const Comp<D>& l, const Comp<D>& g,
                                              const Phys& ph, Comp<D>& b) {
  const double gam = ph.gamma;
  const double unl = dotn<D>(l.u, n);
  const double mn = unl / sqrt(gam * l.p / l.r);
  if (bc == 0) {  // Riemann farfield
    if (fabs(mn) > 1.0) { b = mn < 0.0 ? g : l; return; }
    const double ung = dotn<D>(g.u, n);
    const double rm = ung - 2.0 * sqrt(gam * g.p / g.r) / (gam - 1.0);
    const double rp = unl + 2.0 * sqrt(gam * l.p / l.r) / (gam - 1.0);
    const double unb = 0.5 * (rm + rp);
    const Comp<D>& s = mn < 0.0 ? g : l;
    const double uns = dotn<D>(s.u, n);
#pragma unroll
    for (int k = 0; k < D; ++k) b.u[k] = s.u[k] + (unb - uns) * n[k];
    const double cb = (gam - 1.0) * (rp - rm) / 4.0;
    const double sb = s.p / pow(s.r, gam);
    b.r = pow(cb * cb / (gam * sb), 1.0 / (gam - 1.0));
    b.p = b.r * cb * cb / gam;
    b.e = b.p / ((gam - 1.0) * b.r);
  } else if (bc == 1) {  // velocity inflow
    b = g;
    if (mn > -1.0) b.p = l.p;
  } else if (bc == 2) {  // pressure outflow
    b = l;
    if (mn < 1.0) b.p = g.p;
  } else if (bc == 3) {  // isothermal no-slip wall
    b.r = l.r;
#pragma unroll
    for (int k = 0; k < D; ++k) b.u[k] = g.u[k];
    b.e = g.e;
    b.p = ph.gm1 * b.r * g.e;
  } else if (bc == 4) {  // adiabatic slip wall
    b = l;
#pragma unroll
    for (int k = 0; k < D; ++k) b.u[k] = l.u[k] - unl * n[k];
  } else {  // adiabatic no-slip wall
    b = l;
#pragma unroll
    for (int k = 0; k < D; ++k) b.u[k] = g.u[k];
  }
}

// ---- viscous terms (ViscousFlux.cpp:58-170, VariableConvertor.cpp:574-620, PhysicalModel.cpp:86-165) ----

// Primitive gradient from the conserved gradient g[v*D + k] at a state with velocity u, 1/rho ir and
// total energy per mass Et = E/rho:  grad rho, grad u_m (gu[k][m] = d_k u_m), grad T.
template <int D>
struct PrimGrad {
  double gu[D][D];
  double gT[D];
};

template <int D>
__device__ __forceinline__ void primitiveGradient(const double* g, const double* u, double ir, double Et,
                                                  const Phys& ph, PrimGrad<D>& pg) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double dr = g[k];
    double ge = fma(-dr, Et, g[(D + 1) * D + k]) * ir;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      const double gum = fma(-dr, u[m], g[(1 + m) * D + k]) * ir;
      pg.gu[k][m] = gum;
      ge = fma(-gum, u[m], ge);
    }
    pg.gT[k] = ge * ph.inv_cv;
  }
}

// Dynamic viscosity and thermal conductivity at temperature T (constant or Sutherland,
// PhysicalModel.cpp:86-123): Sutherland ratio sqrt(T^3) (1 + S) / (T + S), S = 110.4 / 273.15.
__device__ __forceinline__ void transport(double T, const Phys& ph, double& mu, double& kappa) {
  if (ph.transport == 2) {
    const double S = 110.4 / 273.15;
    const double r = sqrt(T * T * T) * (1.0 + S) / (T + S);
    mu = ph.mu * r;
    kappa = ph.kappa * r;
  } else {
    mu = ph.mu;
    kappa = ph.kappa;
  }
}

// Viscous stress tau and the energy flux q_k = sum_m tau_km u_m + kappa dT/dx_k.
template <int D>
__device__ __forceinline__ void viscousTensor(const PrimGrad<D>& pg, const double* u, double T, const Phys& ph,
                                              double tau[D][D], double* q) {
  double mu, kappa;
  transport(T, ph, mu, kappa);
  double div = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) div += pg.gu[k][k];
  const double lam = (2.0 / 3.0) * mu * div;
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int m = 0; m < D; ++m) tau[k][m] = mu * (pg.gu[k][m] + pg.gu[m][k]) - (k == m ? lam : 0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double s = kappa * pg.gT[k];
#pragma unroll
    for (int m = 0; m < D; ++m) s = fma(tau[k][m], u[m], s);
    q[k] = s;
  }
}

// Viscous normal flux (0, tau.n, q.n) from velocity u, temperature T and primitive gradient pg.
template <int D>
__device__ __forceinline__ void viscousNormalFlux(const PrimGrad<D>& pg, const double* u, double T, const double* n,
                                                  const Phys& ph, double* f) {
  double tau[D][D], q[D];
  viscousTensor<D>(pg, u, T, ph, tau, q);
  f[0] = 0.0;
#pragma unroll
  for (int m = 0; m < D; ++m) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(tau[k][m], n[k], s);
    f[1 + m] = s;
  }
  f[D + 1] = dotn<D>(q, n);
}

}  // namespace sdg
