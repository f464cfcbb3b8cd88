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
//
// The interior physics (states, convective fluxes, viscous terms) is generic over the scalar type T:
// double is the forward path; the dual numbers of sdg_dual.cuh give its exact derivatives for the
// tangent-linear and adjoint kernels.  The boundary states are double only.
#pragma once
#include <cstdint>

#include "sdg_dual.cuh"

namespace sdg {

struct Phys {
  double gamma, gm1, cv, inv_cv, cp, mu, kappa;
  int transport;  // 1 constant, 2 Sutherland
  double hllc_g2;  // (gamma + 1) / (2 gamma), the HLLC wave-speed factor
  // the reference's incompressible model (IncompresibleEuler/NS with EquationOfState WeakCompressibleFluid,
  // PhysicalModel.cpp:57-78): the last conserved variable is rho e (internal energy), p = c0^2 (rho - rho0) +
  // 0.01 rho0 c0^2, the sound speed is c0
  int incomp;
  double c0, c02, rho0, padd;  // c0, c0^2, rho0, 0.01 rho0 c0^2
  // Boussinesq buoyancy (SourceTerm.cpp:29-58): rho beta (T - Tref) g on the last momentum component, g = 1
  int source;
  double beta, tref;
};

// Reciprocal: rcp.approx.ftz.f64 estimate refined by two Newton-Raphson steps r <- r + r(1 - x r)
// (the classical iteration for 1/x, e.g. P. Markstein, IBM J. Res. Dev. 34(1), 1990).  Each step at
// least doubles the number of correct bits; the result is within a few ulp of 1/x.
__device__ __forceinline__ double rcp(double x) {
  double r;
#ifdef __CUDA_ARCH__
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
#else
  r = 1.0 / x;  // host builds of this header (tests of the pointwise physics)
#endif
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  return r;
}

// -x by flipping the sign bit on the integer pipe (IEEE negation: exact, NaNs and zeros included), keeping
// the stores of the right side's face flux off the FP64 pipe.
__device__ __forceinline__ double negated(double x) {
#ifdef __CUDA_ARCH__
  return __hiloint2double(__double2hiint(x) ^ int(0x80000000u), __double2loint(x));
#else
  return -x;
#endif
}

// Weakly compressible pressure c0^2 (rho - rho0) + padd, in the reference's association: rho - rho0 is exact
// (Sterbenz) for rho within a factor 2 of rho0, so the c0^2 amplification acts on an exact difference.
template <class T>
__device__ __forceinline__ T weakPressure(const T& r, const Phys& ph) {
  return fmaT(ph.c02, r - ph.rho0, ph.padd);
}

template <int D, class T = double>
struct State {
  T r, m[D], E;   // conserved
  T ir, u[D], p;  // 1/rho, velocity, pressure
};

template <int D, class T>
__device__ __forceinline__ void makeState(State<D, T>& s, const T* U, const Phys& ph) {
  s.r = U[0];
#pragma unroll
  for (int k = 0; k < D; ++k) s.m[k] = U[1 + k];
  s.E = U[D + 1];
  s.ir = rcpT(s.r);
  T mu = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) { s.u[k] = s.m[k] * s.ir; mu = fmaT(s.m[k], s.u[k], mu); }
  if constexpr (ScalarTraits<T>::dual) {
    s.p = ph.incomp ? weakPressure(s.r, ph) : ph.gm1 * fmaT(-0.5, mu, s.E);
  } else {
    // one FMA pair serves both models, its operands picked by selects (no FP64 work for the unused model):
    // compressible (gamma - 1)(E - m.u/2) + 0, incompressible c0^2 (rho - rho0) + padd; both round as the
    // separate forms do (fma(a, x, 0) = round(a x), fma(1, r, -rho0) = round(r - rho0))
    const bool inc = ph.incomp;
    const double x = fma(inc ? 1.0 : -0.5, inc ? s.r : mu, inc ? -ph.rho0 : s.E);
    s.p = fma(inc ? ph.c02 : ph.gm1, x, inc ? ph.padd : 0.0);
  }
}

// E + p of the compressible energy flux (E u + p u); the incompressible model transports rho e (no p u).
template <int D, class T>
__device__ __forceinline__ T energyFluxFactor(const State<D, T>& s, const Phys& ph) {
  return ph.incomp ? s.E : s.E + s.p;
}

// Temperature e / cv: compressible e = E/rho - |u|^2/2, incompressible e = (rho e)/rho.
template <int D, class T>
__device__ __forceinline__ T temperatureOf(const State<D, T>& s, const Phys& ph) {
  T u2 = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fmaT(s.u[k], s.u[k], u2);
  return fmaT(ph.incomp ? 0.0 : -0.5, u2, s.E * s.ir) * ph.inv_cv;
}

template <int D, class T>
__device__ __forceinline__ T soundSpeed(const State<D, T>& s, const Phys& ph) {
  return ph.incomp ? T(ph.c0) : sqrtT(ph.gamma * s.p * s.ir);
}

template <int D, class T>
__device__ __forceinline__ T dotn(const T* a, const double* n) {
  T s = a[0] * n[0];
#pragma unroll
  for (int k = 1; k < D; ++k) s = fmaT(a[k], n[k], s);
  return s;
}

template <int D, class T>
__device__ __forceinline__ void normalFlux(const State<D, T>& s, const double* n, T un, T* f, const Phys& ph) {
  f[0] = s.r * un;
#pragma unroll
  for (int k = 0; k < D; ++k) f[1 + k] = fmaT(s.m[k], un, s.p * n[k]);
  f[D + 1] = energyFluxFactor(s, ph) * un;
}

template <int D, class T>
__device__ __forceinline__ void fluxCentral(const State<D, T>& l, const State<D, T>& r, const double* n,
                                            const Phys& ph, T* h) {
  T fl[D + 2], fr[D + 2];
  normalFlux(l, n, dotn<D>(l.u, n), fl, ph);
  normalFlux(r, n, dotn<D>(r.u, n), fr, ph);
#pragma unroll
  for (int i = 0; i < D + 2; ++i) h[i] = 0.5 * (fl[i] + fr[i]);
}

template <int D, class T>
__device__ __forceinline__ void fluxLaxFriedrichs(const State<D, T>& l, const State<D, T>& r, const double* n,
                                                  const Phys& ph, T* h) {
  const T unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  T fl[D + 2], fr[D + 2];
  normalFlux(l, n, unl, fl, ph);
  normalFlux(r, n, unr, fr, ph);
  const T cl = soundSpeed(l, ph), cr = soundSpeed(r, ph);
  const T sr = fmaxT(fabsT(unl) + cl, fabsT(unr) + cr);
  h[0] = 0.5 * fmaT(-sr, r.r - l.r, fl[0] + fr[0]);
#pragma unroll
  for (int k = 0; k < D; ++k) h[1 + k] = 0.5 * fmaT(-sr, r.m[k] - l.m[k], fl[1 + k] + fr[1 + k]);
  h[D + 1] = 0.5 * fmaT(-sr, r.E - l.E, fl[D + 1] + fr[D + 1]);
}

// HLLC with PVRS pressure estimate and Toro's wave-speed factors (ConvectiveFlux.cpp:136-238).
template <int D, class T>
__device__ __forceinline__ void fluxHLLC(const State<D, T>& l, const State<D, T>& r, const double* n, const Phys& ph,
                                         T* h) {
  const T unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  const T gl = ph.gamma * l.ir, gr = ph.gamma * r.ir;  // c^2 = (gamma/rho) p
  const T cl = sqrtT(gl * l.p), cr = sqrtT(gr * r.p);
  const T rhoAvg = 0.5 * (l.r + r.r), cAvg = 0.5 * (cl + cr);
  const T ps = fmaxT(0.0, fmaT(-(unr - unl), rhoAvg * cAvg, 0.5 * (l.p + r.p)));
  const double g2 = ph.hllc_g2;
  // Toro's wave speeds u_n -+ c q with q = sqrt(1 + g2 (ps/p - 1)) where ps > p, else q = 1; there
  // c q = sqrt((gamma/rho) (p + g2 (ps - p))), one square root and no reciprocal.  A real branch (measured:
  // whole warps skip it on smooth flows; the branch-free forms execute more FP64 instructions per face point)
  const T sl = unl - (ps <= l.p ? cl : sqrtT(gl * fmaT(g2, ps - l.p, l.p)));
  if (sl >= 0.0) { normalFlux(l, n, unl, h, ph); return; }
  const T sr = unr + (ps <= r.p ? cr : sqrtT(gr * fmaT(g2, ps - r.p, r.p)));
  if (sr <= 0.0) { normalFlux(r, n, unr, h, ph); return; }
  const T al = l.r * (sl - unl), ar = r.r * (sr - unr);
  const T ss = (r.p - l.p + al * unl - ar * unr) * rcpT(al - ar);
  const bool left = ss >= 0.0;
  const State<D, T>& s = left ? l : r;
  const T sk = left ? sl : sr, un = left ? unl : unr, a = left ? al : ar;
  // h = F(U_k) + S_k (U*_k - U_k) with the reference's star state U*_k = [a, a u + (p* - p) n,
  // a E/rho + p* S* - p u_n] / (S_k - S*), a = rho (S_k - u_n), collected per conserved variable so that
  // neither F(U_k) nor U*_k is formed (18 fewer FP64 instructions per face point; a/rho = S_k - u_n):
  //   rho:  a S*/(S_k - S*)                       (= rho* S*)
  //   m:    m alpha + n (p + A (p* - p))          alpha = (S_k - u_n) S*/(S_k - S*), A = S_k/(S_k - S*)
  //   E:    E alpha + A (p* S* - p u_n) + p u_n   (the last term only with the compressible p u energy flux)
  const T inv = rcpT(sk - ss);
  const T A = sk * inv, ssi = ss * inv;
  const T alpha = (sk - un) * ssi;
  const T beta = fmaT(A, ps - s.p, s.p);
  h[0] = a * ssi;
#pragma unroll
  for (int k = 0; k < D; ++k) h[1 + k] = fmaT(s.m[k], alpha, beta * n[k]);
  const T pu = s.p * un;
  h[D + 1] = fmaT(s.E, alpha, fmaT(A, fmaT(ps, ss, -pu), ph.incomp ? T(0.0) : pu));
}

// Roe flux with Harten's entropy fix, delta = c/20 (ConvectiveFlux.cpp:240-350).
template <int D, class T>
__device__ __forceinline__ void fluxRoe(const State<D, T>& l, const State<D, T>& r, const double* n, const Phys& ph,
                                        T* h) {
  const double g = ph.gamma;
  const T unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  T fl[D + 2], fr[D + 2];
  normalFlux(l, n, unl, fl, ph);
  normalFlux(r, n, unr, fr, ph);
  const T sl = sqrtT(l.r), sr = sqrtT(r.r);
  const T is = rcpT(sl + sr);
  const T wl = sl * is, wr = sr * is;
  const T rho = sl * sr;
  T u[D], u2 = T(0.0), un = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) { u[k] = fmaT(wl, l.u[k], wr * r.u[k]); u2 = fmaT(u[k], u[k], u2); un = fmaT(u[k], n[k], un); }
  // total enthalpy H = (E + p)/rho
  const T hl = (l.E + l.p) * l.ir, hr = (r.E + r.p) * r.ir;
  const T ht = fmaT(wl, hl, wr * hr);
  // c^2 = gamma p / rho with p = (gamma-1) rho e and e = (H - u^2/2)/gamma
  const T c2 = (g - 1.0) * fmaT(-0.5, u2, ht);
  const T c = sqrtT(c2);
  const T ic2 = rcpT(c2);
  const T drho = r.r - l.r, dp = r.p - l.p;
  T du[D], dun = T(0.0), udu = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) { du[k] = r.u[k] - l.u[k]; dun = fmaT(du[k], n[k], dun); udu = fmaT(u[k], du[k], udu); }
  const T delta = c * 0.05;
  const T lm = un - c, lp = un + c;
  const T a1 = fabsT(lm) > delta ? fabsT(lm) : fmaT(lm, lm, delta * delta) * (10.0 * rcpT(c));
  const T a4 = fabsT(lp) > delta ? fabsT(lp) : fmaT(lp, lp, delta * delta) * (10.0 * rcpT(c));
  const T aun = fabsT(un);
  const T rc = rho * c;
  const T s1 = a1 * fmaT(-rc, dun, dp) * (0.5 * ic2);
  const T s2 = aun * fmaT(-dp, ic2, drho);
  const T s3 = aun * rho;
  const T s4 = a4 * fmaT(rc, dun, dp) * (0.5 * ic2);
  const T s14 = s1 + s4, d14 = (s4 - s1) * c;
  h[0] = 0.5 * (fl[0] + fr[0] - (s14 + s2));
#pragma unroll
  for (int k = 0; k < D; ++k)
    h[1 + k] = 0.5 * (fl[1 + k] + fr[1 + k] - fmaT(u[k], s14 + s2, fmaT(d14, n[k], s3 * fmaT(-dun, n[k], du[k]))));
  h[D + 1] = 0.5 * (fl[D + 1] + fr[D + 1] - fmaT(ht, s14, fmaT(d14, un, fmaT(0.5 * u2, s2, s3 * fmaT(-un, dun, udu)))));
}

// Exact flux of the incompressible model (ConvectiveFlux.cpp:352-414): the star state of the two
// characteristic relations with constant sound speed c0,
//   rho* = sqrt(rhoL rhoR exp((unL - unR)/c0)),  un* = (unL + unR)/2 + c0 ln(rhoL/rhoR)/2,
// upwind internal energy (rho e conserved across: e* = e_k rho_k / rho*) and tangential velocity, p* from the
// equation of state; the flux is the normal flux of the star state.
template <int D, class T>
__device__ __forceinline__ void fluxExact(const State<D, T>& l, const State<D, T>& r, const double* n, const Phys& ph,
                                          T* h) {
  const double c0 = ph.c0;
  const T unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  const T rs = sqrtT(l.r * r.r * expT((unl - unr) * (1.0 / c0)));
  const T uns = fmaT(logT(l.r * r.ir), 0.5 * c0, 0.5 * (unl + unr));
  const bool right = uns < 0.0;
  const State<D, T>& k = right ? r : l;
  const T unk = right ? unr : unl;
  const T irs = rcpT(rs);
  const T res = k.E * irs;  // rho* e* = rho_k e_k: conserved internal energy density of the upwind side
  T us[D];
#pragma unroll
  for (int j = 0; j < D; ++j) us[j] = fmaT(uns - unk, n[j], k.u[j]);
  const T ps = weakPressure(rs, ph);
  h[0] = rs * uns;
#pragma unroll
  for (int j = 0; j < D; ++j) h[1 + j] = fmaT(rs * uns, us[j], ps * n[j]);
  h[D + 1] = rs * res * uns;
}

template <int D, int FLUX, class T>
__device__ __forceinline__ void convectiveFlux(const State<D, T>& l, const State<D, T>& r, const double* n,
                                               const Phys& ph, T* h) {
  if constexpr (FLUX == 0) fluxCentral<D>(l, r, n, ph, h);
  else if constexpr (FLUX == 1) fluxLaxFriedrichs<D>(l, r, n, ph, h);
  else if constexpr (FLUX == 2) fluxHLLC<D>(l, r, n, ph, h);
  else if constexpr (FLUX == 3) fluxRoe<D>(l, r, n, ph, h);
  else fluxExact<D>(l, r, n, ph, h);
}

// Computational variables (rho, u, e, p) used by the boundary states; generic over the scalar type like the
// rest of the pointwise physics (double: the forward path; Dual<K>: its derivatives).
template <int D, class T = double>
struct Comp {
  T r, u[D], e, p;
};

template <int D, class T>
__device__ __forceinline__ void compFromState(const State<D, T>& s, Comp<D, T>& c, const Phys& ph) {
  c.r = s.r;
#pragma unroll
  for (int k = 0; k < D; ++k) c.u[k] = s.u[k];
  c.p = s.p;
  if (ph.incomp) { c.e = s.E * s.ir; return; }
  T u2 = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fmaT(s.u[k], s.u[k], u2);
  c.e = fmaT(-0.5, u2, s.E * s.ir);
}

// The last conserved variable of a computational state: rho E (compressible) or rho e (incompressible).
template <int D, class T>
__device__ __forceinline__ T energyOfComp(const Comp<D, T>& c, const Phys& ph) {
  if (ph.incomp) return c.r * c.e;
  T u2 = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) u2 += c.u[k] * c.u[k];
  return c.r * (c.e + 0.5 * u2);
}

template <int D, class T>
__device__ __forceinline__ void normalFluxComp(const Comp<D, T>& c, const double* n, T* f, const Phys& ph) {
  const T un = dotn<D>(c.u, n);
  T u2 = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fmaT(c.u[k], c.u[k], u2);
  f[0] = c.r * un;
#pragma unroll
  for (int k = 0; k < D; ++k) f[1 + k] = fmaT(c.r * un, c.u[k], c.p * n[k]);
  f[D + 1] = ph.incomp ? c.r * c.e * un : fmaT(c.r, fmaT(0.5, u2, c.e), c.p) * un;
}

// Boundary state (BoundaryCondition.cpp:79-547): l = interior trace, g = ghost (user) state.
template <int D, class T>
__device__ __forceinline__ void boundaryState(int bc, const double* n, const Comp<D, T>& l, const Comp<D, T>& g,
                                              const Phys& ph, Comp<D, T>& b) {
  const double gam = ph.gamma;
  const T unl = dotn<D>(l.u, n);
  const T mn = ph.incomp ? unl / ph.c0 : unl / sqrtT(gam * l.p / l.r);
  if (bc == 0) {  // Riemann farfield
    if (fabsT(mn) > 1.0) { b = mn < 0.0 ? g : l; return; }
    if (ph.incomp) {
      // the exact-flux star state between the interior and the ghost (BoundaryCondition.cpp:153-180,243-270)
      const double c0 = ph.c0;
      const T ung = dotn<D>(g.u, n);
      const T rb = sqrtT(l.r * g.r * expT((unl - ung) / c0));
      const T unb = (unl + ung) / 2.0 + logT(l.r / g.r) * c0 / 2.0;
      const Comp<D, T>& s = mn < 0.0 ? g : l;
      const T uns = mn < 0.0 ? ung : unl;
      b.r = rb;
      b.e = s.e * s.r / rb;
#pragma unroll
      for (int k = 0; k < D; ++k) b.u[k] = s.u[k] + (unb - uns) * n[k];
      b.p = weakPressure(rb, ph);
      return;
    }
    const T ung = dotn<D>(g.u, n);
    const T rm = ung - 2.0 * sqrtT(gam * g.p / g.r) / (gam - 1.0);
    const T rp = unl + 2.0 * sqrtT(gam * l.p / l.r) / (gam - 1.0);
    const T unb = 0.5 * (rm + rp);
    const Comp<D, T>& s = mn < 0.0 ? g : l;
    const T uns = dotn<D>(s.u, n);
#pragma unroll
    for (int k = 0; k < D; ++k) b.u[k] = s.u[k] + (unb - uns) * n[k];
    const T cb = (gam - 1.0) * (rp - rm) / 4.0;
    const T sb = s.p / powT(s.r, gam);
    b.r = powT(cb * cb / (gam * sb), 1.0 / (gam - 1.0));
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
    b.p = ph.incomp ? weakPressure(b.r, ph) : ph.gm1 * b.r * g.e;
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
template <int D, class T = double>
struct PrimGrad {
  T gu[D][D];
  T gT[D];
};

// Et = E/rho: total energy per mass (compressible) or internal energy per mass (incompressible, whose
// internal-energy gradient has no -grad(u).u term, VariableConvertor.cpp:598-610).
template <int D, class T>
__device__ __forceinline__ void primitiveGradient(const T* g, const T* u, T ir, T Et, const Phys& ph,
                                                  PrimGrad<D, T>& pg) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const T dr = g[k];
    T ge = fmaT(-dr, Et, g[(D + 1) * D + k]) * ir;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      const T gum = fmaT(-dr, u[m], g[(1 + m) * D + k]) * ir;
      pg.gu[k][m] = gum;
      if (!ph.incomp) ge = fmaT(-gum, u[m], ge);
    }
    pg.gT[k] = ge * ph.inv_cv;
  }
}

// Dynamic viscosity and thermal conductivity at temperature T (constant or Sutherland,
// PhysicalModel.cpp:86-123): Sutherland ratio sqrt(T^3) (1 + S) / (T + S), S = 110.4 / 273.15.
template <class T>
__device__ __forceinline__ void transport(T temp, const Phys& ph, T& mu, T& kappa) {
  if (ph.transport == 2) {
    const double S = 110.4 / 273.15;
    const T r = sqrtT(temp * temp * temp) * (1.0 + S) / (temp + S);
    mu = ph.mu * r;
    kappa = ph.kappa * r;
  } else {
    mu = T(ph.mu);
    kappa = T(ph.kappa);
  }
}

// Viscous stress tau and the energy flux q_k = sum_m tau_km u_m + kappa dT/dx_k.
template <int D, class T>
__device__ __forceinline__ void viscousTensor(const PrimGrad<D, T>& pg, const T* u, T temp, const Phys& ph,
                                              T tau[D][D], T* q) {
  T mu, kappa;
  transport(temp, ph, mu, kappa);
  T div = T(0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) div += pg.gu[k][k];
  const T lam = (2.0 / 3.0) * mu * div;
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int m = 0; m < D; ++m) tau[k][m] = mu * (pg.gu[k][m] + pg.gu[m][k]) - (k == m ? lam : T(0.0));
#pragma unroll
  for (int k = 0; k < D; ++k) {
    T s = kappa * pg.gT[k];
    if (!ph.incomp) {  // incompressible: the internal-energy flux is conduction only (ViscousFlux.cpp:84-101)
#pragma unroll
      for (int m = 0; m < D; ++m) s = fmaT(tau[k][m], u[m], s);
    }
    q[k] = s;
  }
}

// Viscous normal flux (0, tau.n, q.n) from velocity u, temperature T and primitive gradient pg.
template <int D, class T>
__device__ __forceinline__ void viscousNormalFlux(const PrimGrad<D, T>& pg, const T* u, T temp, const double* n,
                                                  const Phys& ph, T* f) {
  T tau[D][D], q[D];
  viscousTensor<D>(pg, u, temp, ph, tau, q);
  f[0] = T(0.0);
#pragma unroll
  for (int m = 0; m < D; ++m) {
    T s = T(0.0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fmaT(tau[k][m], n[k], s);
    f[1 + m] = s;
  }
  f[D + 1] = dotn<D>(q, n);
}

}  // namespace sdg
