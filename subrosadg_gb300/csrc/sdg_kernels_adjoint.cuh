// Tangent-linear (JVP) and adjoint (VJP) kernels of the residual of affine tensor blocks (quadrangles
// P>=2 and hexahedra): compressible and incompressible Euler / Navier-Stokes (BR1, BR2), interior and boundary
// faces, the Boussinesq source.
//
// Forward residual of one stage (nodal Gauss collocation, see sdg_kernels.cuh / sdg_kernels_ns.cuh):
//   Tr = T U                 face traces                       (linear)
//   U+ = P Tr                neighbour traces                  (linear; NS)
//   G  = Grad(U, U+)         BR1 total gradient at the nodes   (linear; NS)
//   Tg = T G                 gradient traces                   (linear; NS)
//   H  = |J_f| [h(UL,UR) - 1/2 (Fv(UL,GL) + Fv(UR,GR)).n]     per face point (nonlinear)
//   Q_b = JA_b . (F(U) - Fv(U,G))                             per node (nonlinear)
//   R  = (1/|J|) [ sum_b Dhat_b Q_b - Lift H ]                 (linear)
// JVP: the linear maps are applied to tangents by the forward kernels themselves (trace pass, exchange,
// gradient kernel); the nonlinear maps here are evaluated in Dual<1> arithmetic.  VJP: the transposed
// linear maps are gathers (a node gathers along its lines, a face point along the line through it), the
// pointwise Jacobians come from Dual<K> passes seeded on the state components, and the viscous flux,
// linear in G, has a hand-written transpose.  The mu-derivative uses that R's viscous part is linear in
// mu (mu and kappa = cp mu / Pr scale together, for the constant and the Sutherland law alike).
#pragma once
#include "sdg_kernels_ns.cuh"

namespace sdg {

// ---- pointwise functions ------------------------------------------------------------------------------

// Contravariant volume fluxes Q[b][v] at a node (the forward stage kernel's formulas).  The viscous
// part is returned separately in Qv (Q includes it), for the mu-derivative.
template <int DIM, bool VISC, class T>
__device__ __forceinline__ void nodeFlux(const T* U, const T* g, const double ja[DIM][DIM], const Phys& ph,
                                         T Q[DIM][DIM + 2], T Qv[DIM][DIM + 2]) {
  constexpr int NV = DIM + 2;
  State<DIM, T> s;
  makeState<DIM>(s, U, ph);
  const T ep = energyFluxFactor(s, ph);
  T tau[DIM][DIM], q[DIM];
  if constexpr (VISC) {
    PrimGrad<DIM, T> pg;
    primitiveGradient<DIM>(g, s.u, s.ir, s.E * s.ir, ph, pg);
    T u2 = T(0.0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) u2 = fmaT(s.u[k], s.u[k], u2);
    viscousTensor<DIM>(pg, s.u, temperatureOf(s, ph), ph, tau, q);
  }
#pragma unroll
  for (int b = 0; b < DIM; ++b) {
    const T vb = dotn<DIM>(s.u, ja[b]);
    Q[b][0] = s.r * vb;
    Qv[b][0] = T(0.0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      T x = fmaT(s.m[k], vb, ja[b][k] * s.p);
      T xv = T(0.0);
      if constexpr (VISC) {
#pragma unroll
        for (int c = 0; c < DIM; ++c) {
          x = fmaT(-ja[b][c], tau[c][k], x);
          xv = fmaT(-ja[b][c], tau[c][k], xv);
        }
      }
      Q[b][1 + k] = x;
      Qv[b][1 + k] = xv;
    }
    T xe = ep * vb;
    T xve = T(0.0);
    if constexpr (VISC) {
      const T qb = dotn<DIM>(q, ja[b]);
      xe = xe - qb;
      xve = -qb;
    }
    Q[b][NV - 1] = xe;
    Qv[b][NV - 1] = xve;
  }
}

// Interior face flux per unit area and its viscous part (the forward face kernels' formulas):
// h = conv(UL, UR) [- 1/2 (fvL + fvR)], hv = the viscous part.
template <int DIM, int FLUX, bool VISC, class T>
__device__ __forceinline__ void faceFluxPoint(const T* ul, const T* ur, const T* gl, const T* gr, const double* n,
                                              const Phys& ph, T* h, T* hv) {
  constexpr int NV = DIM + 2;
  State<DIM, T> l, r;
  makeState<DIM>(l, ul, ph);
  makeState<DIM>(r, ur, ph);
  convectiveFlux<DIM, FLUX>(l, r, n, ph, h);
  if constexpr (VISC) {
    T fl[NV], fr[NV];
    {
      PrimGrad<DIM, T> pg;
      primitiveGradient<DIM>(gl, l.u, l.ir, l.E * l.ir, ph, pg);
      T u2 = T(0.0);
#pragma unroll
      for (int k = 0; k < DIM; ++k) u2 = fmaT(l.u[k], l.u[k], u2);
      viscousNormalFlux<DIM>(pg, l.u, temperatureOf(l, ph), n, ph, fl);
    }
    {
      PrimGrad<DIM, T> pg;
      primitiveGradient<DIM>(gr, r.u, r.ir, r.E * r.ir, ph, pg);
      T u2 = T(0.0);
#pragma unroll
      for (int k = 0; k < DIM; ++k) u2 = fmaT(r.u[k], r.u[k], u2);
      viscousNormalFlux<DIM>(pg, r.u, temperatureOf(r, ph), n, ph, fr);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      hv[v] = -0.5 * (fl[v] + fr[v]);
      h[v] = fmaT(-0.5, fl[v] + fr[v], h[v]);
    }
  } else {
#pragma unroll
    for (int v = 0; v < NV; ++v) hv[v] = T(0.0);
  }
}

// Transpose, with respect to the conserved gradient g[v*D + k], of the viscous fluxes Fv_c (direction c)
// at a state (U fixed):  lamg += sum_c (dFv_c/dg)^T lamF[c].
template <int D>
__device__ __forceinline__ void viscousTransposeG(const double* U, const Phys& ph, const double lamF[D][D + 2],
                                                  double* lamg) {
  constexpr int NV = D + 2;
  State<D> s;
  makeState<D>(s, U, ph);
  double u2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) u2 = fma(s.u[k], s.u[k], u2);
  const double Et = s.E * s.ir;
  const double temp = fma(-0.5, u2, Et) * ph.inv_cv;
  double mu, kappa;
  transport(temp, ph, mu, kappa);
  double lt[D][D], lgT[D];
#pragma unroll
  for (int c = 0; c < D; ++c) {
#pragma unroll
    for (int m = 0; m < D; ++m) lt[c][m] = fma(lamF[c][NV - 1], s.u[m], lamF[c][1 + m]);
    lgT[c] = kappa * lamF[c][NV - 1];
  }
  double tr = 0.0;
#pragma unroll
  for (int j = 0; j < D; ++j) tr += lt[j][j];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double lge = ph.inv_cv * lgT[k];
    double ldr = -Et * s.ir * lge;
    lamg[(D + 1) * D + k] += s.ir * lge;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      double lgu = mu * (lt[k][m] + lt[m][k]);
      if (k == m) lgu -= (2.0 / 3.0) * mu * tr;
      const double lgum = fma(-s.u[m], lge, lgu);
      lamg[(1 + m) * D + k] += s.ir * lgum;
      ldr = fma(-s.u[m] * s.ir, lgum, ldr);
    }
    lamg[k] += ldr;
  }
}


// ---- dual-number transposes (the incompressible model and the Boussinesq source) -----------------------
// Volume: lamU = sum_b (dQ_b/dU)^T lq[b] + lam_S dS/dU (S the buoyancy on the last momentum component),
// lamG = sum_b (dQ_b/dG)^T lq[b]; returns sum_b lq[b] . Qv_b (the viscosity term).  Used only by the GEN
// instantiations, so the compressible kernels keep their hand-written sweeps and register allocation.
template <int DIM, bool VISC>
__device__ __forceinline__ double volumeReverseGeneric(const double* U, const double* G, const double (*ja)[DIM],
                                                    const double (*lq)[DIM + 2], double lamS, const Phys& ph,
                                                    double* lamU, double* lamG) {
  constexpr int NV = DIM + 2, NG = NV * DIM;
  using DK = Dual<NV>;
  double mupart = 0.0;
  {
    DK x[NV], g[VISC ? NG : 1], Q[DIM][NV], Qv[DIM][NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) { x[v] = DK(U[v]); x[v].d[v] = 1.0; }
    if constexpr (VISC) {
#pragma unroll
      for (int c = 0; c < NG; ++c) g[c] = DK(G[c]);
    }
    nodeFlux<DIM, VISC>(x, g, ja, ph, Q, Qv);
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lq[b][v], Q[b][v].d[w], acc);
      lamU[w] = acc;
    }
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) mupart = fma(lq[b][v], Qv[b][v].v, mupart);
    if (ph.source) {
      State<DIM, DK> st;
      makeState<DIM>(st, x, ph);
      const DK S = st.r * ph.beta * (temperatureOf(st, ph) - ph.tref);
#pragma unroll
      for (int w = 0; w < NV; ++w) lamU[w] = fma(lamS, S.d[w], lamU[w]);
    }
  }
  if constexpr (VISC) {
    using DG = Dual<NG>;
    DG x[NV], g[NG], Q[DIM][NV], Qv[DIM][NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) x[v] = DG(U[v]);
#pragma unroll
    for (int c = 0; c < NG; ++c) { g[c] = DG(G[c]); g[c].d[c] = 1.0; }
    nodeFlux<DIM, VISC>(x, g, ja, ph, Q, Qv);
#pragma unroll
    for (int c = 0; c < NG; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lq[b][v], Q[b][v].d[c], acc);
      lamG[c] = acc;
    }
  }
  return mupart;
}

// Face: one side's viscous flux enters h as -1/2 Fv(U, G).n; lamU += its transpose in U, lamG = in G;
// returns the viscosity term sum_v lh[v] (-1/2 Fv.n)(v).
template <int DIM>
__device__ __forceinline__ double faceViscousReverseGeneric(const double* U, const double* G, const double* n,
                                                         const double* lh, const Phys& ph, double* lamU,
                                                         double* lamG) {
  constexpr int NV = DIM + 2, NG = NV * DIM;
  double mupart = 0.0;
  {
    using DK = Dual<NV>;
    DK x[NV], g[NG], f[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) { x[v] = DK(U[v]); x[v].d[v] = 1.0; }
#pragma unroll
    for (int c = 0; c < NG; ++c) g[c] = DK(G[c]);
    State<DIM, DK> s;
    makeState<DIM>(s, x, ph);
    PrimGrad<DIM, DK> pg;
    primitiveGradient<DIM>(g, s.u, s.ir, s.E * s.ir, ph, pg);
    viscousNormalFlux<DIM>(pg, s.u, temperatureOf(s, ph), n, ph, f);
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double acc = 0.0;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc = fma(lh[v], f[v].d[w], acc);
      lamU[w] = fma(-0.5, acc, lamU[w]);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) mupart = fma(-0.5 * lh[v], f[v].v, mupart);
  }
  {
    using DG = Dual<NG>;
    DG x[NV], g[NG], f[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) x[v] = DG(U[v]);
#pragma unroll
    for (int c = 0; c < NG; ++c) { g[c] = DG(G[c]); g[c].d[c] = 1.0; }
    State<DIM, DG> s;
    makeState<DIM>(s, x, ph);
    PrimGrad<DIM, DG> pg;
    primitiveGradient<DIM>(g, s.u, s.ir, s.E * s.ir, ph, pg);
    viscousNormalFlux<DIM>(pg, s.u, temperatureOf(s, ph), n, ph, f);
#pragma unroll
    for (int c = 0; c < NG; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc = fma(lh[v], f[v].d[c], acc);
      lamG[c] = -0.5 * acc;
    }
  }
  return mupart;
}

// ---- hand-written reverse sweeps (adjoints of the forward formulas, line by line) ---------------------
// Euler contravariant volume fluxes Q_b = (rho vb, m vb + ja_b p, (E + p) vb), vb = u . ja_b:
// lamU = sum_b (dQ_b/dU)^T lq[b].
template <int D>
__device__ __forceinline__ void eulerVolumeReverse(const double* U, const double ja[D][D], const double lq[D][D + 2],
                                                   const Phys& ph, double* lamU) {
  constexpr int NV = D + 2;
  const double rho = U[0], E = U[D + 1];
  const double ir = rcp(rho);
  double u[D], mu2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { u[k] = U[1 + k] * ir; mu2 = fma(U[1 + k], u[k], mu2); }
  const double p = ph.gm1 * fma(-0.5, mu2, E), ep = E + p;
  double lrho = 0.0, lE = 0.0, lp = 0.0, lm[D], lu[D];
#pragma unroll
  for (int k = 0; k < D; ++k) { lm[k] = 0.0; lu[k] = 0.0; }
#pragma unroll
  for (int b = 0; b < D; ++b) {
    double vb = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) vb = fma(u[k], ja[b][k], vb);
    double lvb = fma(lq[b][0], rho, lq[b][NV - 1] * ep);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      lvb = fma(lq[b][1 + k], U[1 + k], lvb);
      lp = fma(lq[b][1 + k], ja[b][k], lp);
      lm[k] = fma(lq[b][1 + k], vb, lm[k]);
    }
    lp = fma(lq[b][NV - 1], vb, lp);
    lrho = fma(lq[b][0], vb, lrho);
    lE = fma(lq[b][NV - 1], vb, lE);
#pragma unroll
    for (int k = 0; k < D; ++k) lu[k] = fma(lvb, ja[b][k], lu[k]);
  }
  lE = fma(ph.gm1, lp, lE);
  const double hp = -0.5 * ph.gm1 * lp;
  double lir = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lm[k] = fma(hp, u[k], lm[k]);
    lu[k] = fma(hp, U[1 + k], lu[k]);
    lm[k] = fma(lu[k], ir, lm[k]);
    lir = fma(lu[k], U[1 + k], lir);
  }
  lrho = fma(-ir * ir, lir, lrho);
  lamU[0] = lrho;
#pragma unroll
  for (int k = 0; k < D; ++k) lamU[1 + k] = lm[k];
  lamU[NV - 1] = lE;
}

// Viscous fluxes Fv_c (direction c) = (0, tau[c][.], q[c]) at state U with conserved gradient g:
// lamU += (dFv/dU)^T lamF, lamg += (dFv/dg)^T lamF, and the return value is sum_c lamF[c] . Fv_c
// (the mu-derivative term: Fv is proportional to the reference viscosity).
template <int D>
__device__ __forceinline__ double viscousReverse(const double* U, const double* g, const double lamF[D][D + 2],
                                                 const Phys& ph, double* lamU, double* lamg) {
  constexpr int NV = D + 2;
  const double rho = U[0], E = U[D + 1];
  const double ir = rcp(rho);
  double u[D], u2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { u[k] = U[1 + k] * ir; u2 = fma(u[k], u[k], u2); }
  const double Et = E * ir;
  const double temp = fma(-0.5, u2, Et) * ph.inv_cv;
  double mu, kappa;
  transport(temp, ph, mu, kappa);
  double dr[D], B[D], A[D][D], gum[D][D], gT[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    dr[k] = g[k];
    B[k] = fma(-dr[k], Et, g[(D + 1) * D + k]);
    double ge = B[k] * ir;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      A[k][m] = fma(-dr[k], u[m], g[(1 + m) * D + k]);
      gum[k][m] = A[k][m] * ir;
      ge = fma(-gum[k][m], u[m], ge);
    }
    gT[k] = ge * ph.inv_cv;
  }
  double div = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) div += gum[k][k];
  double tau[D][D], q[D];
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int m = 0; m < D; ++m) tau[k][m] = mu * (gum[k][m] + gum[m][k]) - (k == m ? (2.0 / 3.0) * mu * div : 0.0);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double s = kappa * gT[k];
#pragma unroll
    for (int m = 0; m < D; ++m) s = fma(tau[k][m], u[m], s);
    q[k] = s;
  }
  // value term
  double fdot = 0.0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
#pragma unroll
    for (int m = 0; m < D; ++m) fdot = fma(lamF[c][1 + m], tau[c][m], fdot);
    fdot = fma(lamF[c][NV - 1], q[c], fdot);
  }
  // reverse: q[c] = kappa gT[c] + sum_m tau[c][m] u[m]
  double lt[D][D], lu[D], lgT[D], lkappa = 0.0;
#pragma unroll
  for (int m = 0; m < D; ++m) lu[m] = 0.0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const double le = lamF[c][NV - 1];
#pragma unroll
    for (int m = 0; m < D; ++m) {
      lt[c][m] = fma(le, u[m], lamF[c][1 + m]);
      lu[m] = fma(le, tau[c][m], lu[m]);
    }
    lgT[c] = kappa * le;
    lkappa = fma(le, gT[c], lkappa);
  }
  // tau = mu (gum + gum^T) - 2/3 mu div I
  double tr = 0.0, lmu = 0.0;
#pragma unroll
  for (int j = 0; j < D; ++j) tr += lt[j][j];
#pragma unroll
  for (int k = 0; k < D; ++k)
#pragma unroll
    for (int m = 0; m < D; ++m)
      lmu = fma(lt[k][m], gum[k][m] + gum[m][k] - (k == m ? (2.0 / 3.0) * div : 0.0), lmu);
  double lir = 0.0, lEt = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const double lge = ph.inv_cv * lgT[k];
    lamg[(D + 1) * D + k] = fma(ir, lge, lamg[(D + 1) * D + k]);
    lir = fma(B[k], lge, lir);
    lEt = fma(-dr[k] * ir, lge, lEt);
    double ldr = -Et * ir * lge;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      double lg = mu * (lt[k][m] + lt[m][k]);
      if (k == m) lg -= (2.0 / 3.0) * mu * tr;
      lg = fma(-u[m], lge, lg);              // ge contains -gum[k][m] u[m]
      lu[m] = fma(-gum[k][m], lge, lu[m]);
      lamg[(1 + m) * D + k] = fma(ir, lg, lamg[(1 + m) * D + k]);
      ldr = fma(-u[m] * ir, lg, ldr);
      lir = fma(lg, A[k][m], lir);
      lu[m] = fma(-dr[k] * ir, lg, lu[m]);
    }
    lamg[k] += ldr;
  }
  // transport law: Sutherland mu = mu0 r(T), kappa = kappa0 r(T), r'(T) = r (3/(2T) - 1/(T+S))
  if (ph.transport == 2) {
    const double S = 110.4 / 273.15;
    const double r = sqrt(temp * temp * temp) * (1.0 + S) / (temp + S);
    const double dr_dT = r * (1.5 / temp - 1.0 / (temp + S));
    const double lT = (lmu * ph.mu + lkappa * ph.kappa) * dr_dT;
    lEt = fma(ph.inv_cv, lT, lEt);
#pragma unroll
    for (int m = 0; m < D; ++m) lu[m] = fma(-ph.inv_cv * lT, u[m], lu[m]);
  }
  // Et = E ir, u = m ir, ir = 1/rho
  lamU[NV - 1] = fma(ir, lEt, lamU[NV - 1]);
  lir = fma(E, lEt, lir);
#pragma unroll
  for (int m = 0; m < D; ++m) {
    lamU[1 + m] = fma(ir, lu[m], lamU[1 + m]);
    lir = fma(U[1 + m], lu[m], lir);
  }
  lamU[0] = fma(-ir * ir, lir, lamU[0]);
  return fdot;
}

// Roe flux with Harten's entropy fix (fluxRoe): lamL += (dh/dUL)^T lh, lamR += (dh/dUR)^T lh.
template <int D>
__device__ __forceinline__ void roeReverse(const double* UL, const double* UR, const double* n, const Phys& ph,
                                           const double* lh, double* lamL, double* lamR) {
  constexpr int NV = D + 2;
  State<D> l, r;
  makeState<D>(l, UL, ph);
  makeState<D>(r, UR, ph);
  const double g = ph.gamma;
  const double unl = dotn<D>(l.u, n), unr = dotn<D>(r.u, n);
  const double sl = sqrt(l.r), sr = sqrt(r.r);
  const double is = rcp(sl + sr);
  const double wl = sl * is, wr = sr * is;
  const double rho = sl * sr;
  double u[D], u2 = 0.0, un = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { u[k] = fma(wl, l.u[k], wr * r.u[k]); u2 = fma(u[k], u[k], u2); un = fma(u[k], n[k], un); }
  const double hl = (l.E + l.p) * l.ir, hr = (r.E + r.p) * r.ir;
  const double ht = fma(wl, hl, wr * hr);
  const double c2 = (g - 1.0) * fma(-0.5, u2, ht);
  const double c = sqrt(c2);
  const double ic2 = rcp(c2);
  const double ic = rcp(c);
  const double drho = r.r - l.r, dp = r.p - l.p;
  double du[D], dun = 0.0, udu = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) { du[k] = r.u[k] - l.u[k]; dun = fma(du[k], n[k], dun); udu = fma(u[k], du[k], udu); }
  const double delta = c * 0.05;
  const double lmv = un - c, lpv = un + c;
  const bool e1 = fabs(lmv) > delta, e4 = fabs(lpv) > delta;
  const double a1 = e1 ? fabs(lmv) : fma(lmv, lmv, delta * delta) * (10.0 * ic);
  const double a4 = e4 ? fabs(lpv) : fma(lpv, lpv, delta * delta) * (10.0 * ic);
  const double aun = fabs(un);
  const double rc = rho * c;
  const double X1 = fma(-rc, dun, dp), X4 = fma(rc, dun, dp), h2 = 0.5 * ic2;
  const double s1 = a1 * X1 * h2, s4 = a4 * X4 * h2;
  const double s2 = aun * fma(-dp, ic2, drho);
  const double s3 = aun * rho;
  const double s14 = s1 + s4, d14 = (s4 - s1) * c;
  // h = 1/2 (fl + fr) - 1/2 Diss: cotangents of the dissipation terms
  double mk[D];
  const double m0 = -0.5 * lh[0], mE = -0.5 * lh[NV - 1];
#pragma unroll
  for (int k = 0; k < D; ++k) mk[k] = -0.5 * lh[1 + k];
  double mu_u = 0.0, mu_n = 0.0, mu_dd = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    mu_u = fma(mk[k], u[k], mu_u);
    mu_n = fma(mk[k], n[k], mu_n);
    mu_dd = fma(mk[k], fma(-dun, n[k], du[k]), mu_dd);
  }
  const double ls14 = m0 + mu_u + mE * ht;
  const double ls2 = m0 + mu_u + mE * 0.5 * u2;
  const double ld14 = fma(mE, un, mu_n);
  const double ls3 = fma(mE, fma(-un, dun, udu), mu_dd);
  double lu[D], ldu[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lu[k] = fma(mk[k], s14 + s2, mE * s3 * du[k]);
    ldu[k] = fma(mk[k], s3, mE * s3 * u[k]);
  }
  double lu2 = mE * 0.5 * s2;
  double lht = mE * s14;
  double lun = mE * fma(-s3, dun, d14);
  double ldun = -s3 * fma(mE, un, mu_n);
  double ls1 = fma(-ld14, c, ls14), ls4 = fma(ld14, c, ls14);
  double lc = ld14 * (s4 - s1);
  const double la1 = ls1 * X1 * h2, la4 = ls4 * X4 * h2;
  const double lX1 = ls1 * a1 * h2, lX4 = ls4 * a4 * h2;
  const double lh2 = fma(ls1 * a1, X1, ls4 * a4 * X4);
  double ldp = lX1 + lX4;
  double lrc = (lX4 - lX1) * dun;
  ldun = fma(lX4 - lX1, rc, ldun);
  double lic2 = 0.5 * lh2;
  double laun = ls2 * fma(-dp, ic2, drho);
  double ldrho = ls2 * aun;
  ldp = fma(-ls2 * aun, ic2, ldp);
  lic2 = fma(-ls2 * aun, dp, lic2);
  laun = fma(ls3, rho, laun);
  double lrho = ls3 * aun;
  lrho = fma(lrc, c, lrho);
  lc = fma(lrc, rho, lc);
  lun += un < 0.0 ? -laun : laun;
  double llm, llp, ldelta = 0.0;
  if (e1) { llm = lmv < 0.0 ? -la1 : la1; }
  else {
    llm = la1 * 2.0 * lmv * 10.0 * ic;
    ldelta = fma(la1 * 2.0 * delta, 10.0 * ic, ldelta);
    lc = fma(-la1 * fma(lmv, lmv, delta * delta), 10.0 * ic * ic, lc);
  }
  if (e4) { llp = lpv < 0.0 ? -la4 : la4; }
  else {
    llp = la4 * 2.0 * lpv * 10.0 * ic;
    ldelta = fma(la4 * 2.0 * delta, 10.0 * ic, ldelta);
    lc = fma(-la4 * fma(lpv, lpv, delta * delta), 10.0 * ic * ic, lc);
  }
  lun += llm + llp;
  lc += llp - llm + 0.05 * ldelta;
  const double lc2 = lc * 0.5 * ic - lic2 * ic2 * ic2;
  lht = fma(g - 1.0, lc2, lht);
  lu2 = fma(-0.5 * (g - 1.0), lc2, lu2);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lu[k] = fma(2.0 * u[k], lu2, fma(n[k], lun, lu[k]));
    ldu[k] = fma(n[k], ldun, ldu[k]);
  }
  // left / right primitive cotangents
  double llu[D], lru[D];
  double llr = -ldrho, lrr = ldrho, llp_ = -ldp, lrp_ = ldp;
  const double lwl0 = lht * hl, lhl = lht * wl, lwr0 = lht * hr, lhr = lht * wr;
  double lwl = lwl0, lwr = lwr0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    llu[k] = fma(lu[k], wl, -ldu[k]);
    lru[k] = fma(lu[k], wr, ldu[k]);
    lwl = fma(lu[k], l.u[k], lwl);
    lwr = fma(lu[k], r.u[k], lwr);
  }
  double lsl = fma(lrho, sr, lwl * is), lsr = fma(lrho, sl, lwr * is);
  const double lsum = -is * is * fma(lwl, sl, lwr * sr);
  lsl += lsum; lsr += lsum;
  llr = fma(lsl, 0.5 * rcp(sl), llr);
  lrr = fma(lsr, 0.5 * rcp(sr), lrr);
  double lLE = lhl * l.ir, lRE = lhr * r.ir;
  llp_ = fma(lhl, l.ir, llp_);
  lrp_ = fma(lhr, r.ir, lrp_);
  double lLir = lhl * (l.E + l.p), lRir = lhr * (r.E + r.p);
  // 1/2 (fl + fr): normal fluxes of each side
  double gk[D];
  const double g0 = 0.5 * lh[0], gE = 0.5 * lh[NV - 1];
#pragma unroll
  for (int k = 0; k < D; ++k) gk[k] = 0.5 * lh[1 + k];
  double lunl = fma(g0, l.r, gE * (l.E + l.p)), lunr = fma(g0, r.r, gE * (r.E + r.p));
  double lLm[D], lRm[D], gn = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lunl = fma(gk[k], l.m[k], lunl);
    lunr = fma(gk[k], r.m[k], lunr);
    lLm[k] = gk[k] * unl;
    lRm[k] = gk[k] * unr;
    gn = fma(gk[k], n[k], gn);
  }
  llr = fma(g0, unl, llr);
  lrr = fma(g0, unr, lrr);
  llp_ += fma(gE, unl, gn);
  lrp_ += fma(gE, unr, gn);
  lLE = fma(gE, unl, lLE);
  lRE = fma(gE, unr, lRE);
#pragma unroll
  for (int k = 0; k < D; ++k) { llu[k] = fma(n[k], lunl, llu[k]); lru[k] = fma(n[k], lunr, lru[k]); }
  // states: p = gm1 (E - 1/2 m.u), u = m ir, ir = 1/rho
  lLE = fma(ph.gm1, llp_, lLE);
  lRE = fma(ph.gm1, lrp_, lRE);
  const double hpl = -0.5 * ph.gm1 * llp_, hpr = -0.5 * ph.gm1 * lrp_;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lLm[k] = fma(hpl, l.u[k], lLm[k]);
    llu[k] = fma(hpl, l.m[k], llu[k]);
    lRm[k] = fma(hpr, r.u[k], lRm[k]);
    lru[k] = fma(hpr, r.m[k], lru[k]);
    lLm[k] = fma(llu[k], l.ir, lLm[k]);
    lRm[k] = fma(lru[k], r.ir, lRm[k]);
    lLir = fma(llu[k], l.m[k], lLir);
    lRir = fma(lru[k], r.m[k], lRir);
  }
  llr = fma(-l.ir * l.ir, lLir, llr);
  lrr = fma(-r.ir * r.ir, lRir, lrr);
  lamL[0] += llr; lamR[0] += lrr;
#pragma unroll
  for (int k = 0; k < D; ++k) { lamL[1 + k] += lLm[k]; lamR[1 + k] += lRm[k]; }
  lamL[NV - 1] += lLE; lamR[NV - 1] += lRE;
}

// ---- work buffers -------------------------------------------------------------------------------------
struct AdjArgs {
  const double* u;        // stage input state [e][USTRIDE]
  const double* geom;     // [e][d*d+1]
  const double* tables;   // TensorTables
  const double* grad;     // NS: forward gradient at the nodes [e][nv*d][NB]
  const double* face;     // forward traces of u [slot][nv][nfq]
  const double* faceGrad; // NS: forward gradient traces [slot][nv*d][nfq]
  const int* conn;        // interior faces (slot L, slot R, rotation)
  const double* fgeo;     // per face (n, |J_f|)
  // tangent-linear
  const double* du;       // tangent of u (stage input) [e][USTRIDE]
  const double* dgrad;    // NS: tangent of the gradient [e][nv*d][NB]
  const double* dface;    // tangent traces [slot][nv][nfq]
  const double* dfaceGrad;// NS: tangent gradient traces
  double* dflux;          // tangent face flux |J_f| dH [slot][nv][nfq]
  double dmu;             // tangent of the viscosity
  // RK / outputs of the tangent element kernel
  const double* dbase;    // tangent of the step's base state
  double* dout;           // tangent of the new state (or null)
  double* drate;          // tangent of du/dt at the nodes (or null) [e][USTRIDE]
  double* dtrace;         // traces of dout [slot][nv][nfq] (or null)
  double c0, c1, c2dt;
  // adjoint
  const double* lam;      // cotangent of du/dt (VJP input) [e][USTRIDE]
  double* lamU;           // cotangent of u [e][USTRIDE]
  double* lamG;           // NS: cotangent of the node gradient [e][nv*d][NB]
  double* lamH;           // cotangent of the face flux slots [slot][nv][nfq]
  double* lamTr;          // cotangent of the traces [slot][nv][nfq]
  double* lamTg;          // NS: cotangent of the gradient traces [slot][nv*d][nfq]
  double* lamUp;          // NS: cotangent of the neighbour traces [slot][nv][nfq]
  double* muPart;         // per-tile partial sums of <lambda, dR/dmu> * mu
  // RK combination of the adjoint element kernel:  stage = c1 lamIn + c2dt VJP, base += c0 lamIn
  const double* lamIn;
  double* lamStage;
  double* lamBase;
  int accumulateAll;      // stage 0 in reverse: base += c0 lamIn + c1 lamIn + c2dt VJP (stage unused)
  unsigned* status;
  int64_t ne, faceBase, nface;
  int n1d, epb;           // n1d < 0: triangular faces paired through perm
  const int* perm;        // triangular faces: [3][nfq] right point of left point j at rotation r
  // boundary faces: ghost states [face][j][rho, u, e, p]; cotangent of each boundary point's ghost
  // primitive (rho, u, T), accumulated with weight ghostScale; NS: the tangent of the neighbour traces
  double* dother;
  const double* ghost;
  double* lamGhost;
  double ghostScale;
  const double* fmetric;  // outward n|J_f| of each local face [e][NF][d], or of each face point [e][NF][nfq][d]
  int fgeoPoint;          // 1: fgeo per face point [face][j][n, |J_f|] (curved meshes, non-parallelepiped hexahedra)
  int fmetricPoint;       // 1: fmetric per face point
};

// ---- surface force (the reference's View force, VariableConvertor.cpp:883-906, Paraview.cpp:99-106) ------
// Per boundary point of the selected faces: w_j |J_f| (p n - tau n) from the interior trace (and, for
// Navier-Stokes, its gradient trace); n points out of the fluid.
struct ForceArgs {
  const double* face;       // traces [slot][nv][nfq]
  const double* faceGrad;   // Navier-Stokes gradient traces [slot][nv*d][nfq] (or null)
  const int* conn;          // boundary (slot, condition, 0)
  const double* fgeo;       // boundary (n, |J_f|)
  const int* select;        // [face] 1 for the faces of the group
  const double* fw;         // face-rule weights [nfq]
  double* out;              // force: [point][d]; cotangent: the trace cotangent slots [slot][nv][nfq]
  double dir[3];            // cotangent: the direction of the force component
  int64_t nface;
  int n1d, ns;
  int fgeoPoint, pad;       // 1: fgeo per face point (curved meshes)
};

template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) surfaceForceKernel(ForceArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  const int nfq = nfqOf<DIM>(a.n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  double* out = a.out + t * DIM;
  if (!a.select[f]) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) out[k] = 0.0;
    return;
  }
  const int64_t L = int64_t(a.conn[f * 3]) * NV * nfq + j;
  double ul[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = a.face[L + v * nfq];
  State<DIM> s;
  makeState<DIM>(s, ul, ph);
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double wa = a.fw[j] * fg[3];
  double tn[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) tn[k] = 0.0;
  if (a.ns) {
    const int64_t LG = int64_t(a.conn[f * 3]) * NV * DIM * nfq + j;
    double g[NV * DIM];
#pragma unroll
    for (int c = 0; c < NV * DIM; ++c) g[c] = a.faceGrad[LG + c * nfq];
    PrimGrad<DIM> pg;
    primitiveGradient<DIM>(g, s.u, s.ir, s.E * s.ir, ph, pg);
    double tau[DIM][DIM], q[DIM];
    viscousTensor<DIM>(pg, s.u, temperatureOf(s, ph), ph, tau, q);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int m = 0; m < DIM; ++m) tn[k] = fma(tau[k][m], n[m], tn[k]);
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) out[k] = wa * fma(s.p, n[k], -tn[k]);
}

// dir . (p n - tau n) at a boundary point from its trace and (Navier-Stokes) gradient trace, generic.
template <int DIM, class T>
__device__ __forceinline__ T forceDotOf(const T* ul, const T* gr, const double* n, const double* dir, bool ns,
                                        const Phys& ph) {
  State<DIM, T> s;
  makeState<DIM>(s, ul, ph);
  double nd = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) nd = fma(n[k], dir[k], nd);
  T out = s.p * nd;
  if (ns) {
    PrimGrad<DIM, T> pg;
    primitiveGradient<DIM>(gr, s.u, s.ir, s.E * s.ir, ph, pg);
    T tau[DIM][DIM], q[DIM];
    viscousTensor<DIM>(pg, s.u, temperatureOf(s, ph), ph, tau, q);
#pragma unroll
    for (int k = 0; k < DIM; ++k)
#pragma unroll
      for (int m = 0; m < DIM; ++m) out = out - dir[k] * tau[k][m] * n[m];
  }
  return out;
}

// Cotangent of the direction component of the force with respect to the interior traces (and, Navier-Stokes,
// the gradient traces) of the selected boundary points; zero elsewhere (the slots are boundary-owned).
// out: trace slots [slot][nv][nfq]; outG: gradient-trace slots [slot][nv*d][nfq].
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) surfaceForceTraceCotangentKernel(ForceArgs a, Phys ph, double* outG) {
  constexpr int NV = DIM + 2, NG = NV * DIM;
  using DK = Dual<NV>;
  using DG = Dual<NG>;
  const int nfq = nfqOf<DIM>(a.n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int64_t L = int64_t(a.conn[f * 3]) * NV * nfq + j, LG = int64_t(a.conn[f * 3]) * NG * nfq + j;
  double n[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  const double scale = a.select[f] ? a.fw[j] * faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3] : 0.0;
  double ul[NV], gg[NG];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = a.face[L + v * nfq];
#pragma unroll
  for (int c = 0; c < NG; ++c) gg[c] = a.ns ? a.faceGrad[LG + c * nfq] : 0.0;
  {
    DK x[NV], gr[NG];
#pragma unroll
    for (int v = 0; v < NV; ++v) { x[v] = DK(ul[v]); x[v].d[v] = 1.0; }
#pragma unroll
    for (int c = 0; c < NG; ++c) gr[c] = DK(gg[c]);
    const DK J = forceDotOf<DIM>(x, gr, n, a.dir, a.ns != 0, ph);
#pragma unroll
    for (int v = 0; v < NV; ++v) a.out[L + v * nfq] = scale * J.d[v];
  }
  if (a.ns) {
    DG x[NV], gr[NG];
#pragma unroll
    for (int v = 0; v < NV; ++v) x[v] = DG(ul[v]);
#pragma unroll
    for (int c = 0; c < NG; ++c) { gr[c] = DG(gg[c]); gr[c].d[c] = 1.0; }
    const DG J = forceDotOf<DIM>(x, gr, n, a.dir, true, ph);
#pragma unroll
    for (int c = 0; c < NG; ++c) outG[LG + c * nfq] = scale * J.d[c];
  }
}

// ---- boundary faces (Euler) -------------------------------------------------------------------------
// Boundary flux |J_f| F(U_b(U_L, g)).n (SpatialDiscrete.cpp:750-842): the tangent in the interior trace, and
// its transpose to the trace and to the ghost primitive (rho, u, T) of the point, e = cv T and p from the
// equation of state as the ghost states are built (VariableConvertor.cpp:341-380).
template <int DIM, class T>
__device__ __forceinline__ void boundaryFluxOf(const T* ul, const T* gprim, const double* n, int bc, const Phys& ph,
                                               T* h) {
  State<DIM, T> s;
  makeState<DIM>(s, ul, ph);
  Comp<DIM, T> l, g, b;
  compFromState<DIM>(s, l, ph);
  g.r = gprim[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gprim[1 + k];
  g.e = ph.cv * gprim[DIM + 1];
  g.p = ph.incomp ? weakPressure(g.r, ph) : ph.gm1 * g.r * g.e;
  boundaryState<DIM>(bc, n, l, g, ph, b);
  normalFluxComp<DIM>(b, n, h, ph);
}

template <int DIM>
__device__ __forceinline__ void ghostPrimitiveOf(const double* ghost, int64_t point, const Phys& ph, double* gp) {
  const double* g = ghost + point * (DIM + 3);
  gp[0] = g[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) gp[1 + k] = g[1 + k];
  gp[DIM + 1] = g[DIM + 1] * ph.inv_cv;
}

__device__ __forceinline__ void blockSum(double x, double* part, double* sRed);

// Navier-Stokes boundary flux (faceNSBoundaryPoint's arithmetic, generic): convective flux of the boundary
// state minus the average of the viscous fluxes of (walls: the wall state; else the interior) and of the
// boundary state, both with the interior primitive gradient (adiabatic walls: no temperature gradient on the
// boundary side).  hv = the viscous part (linear in the viscosity).
template <int DIM, class T>
__device__ __forceinline__ void boundaryNSFluxOf(const T* ul, const T* gr, const T* gprim, const double* n, int bc,
                                                 const Phys& ph, T* h, T* hv) {
  constexpr int NV = DIM + 2;
  State<DIM, T> s;
  makeState<DIM>(s, ul, ph);
  Comp<DIM, T> l, g, b;
  compFromState<DIM>(s, l, ph);
  g.r = gprim[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gprim[1 + k];
  g.e = ph.cv * gprim[DIM + 1];
  g.p = ph.incomp ? weakPressure(g.r, ph) : ph.gm1 * g.r * g.e;
  boundaryState<DIM>(bc, n, l, g, ph, b);
  normalFluxComp<DIM>(b, n, h, ph);
  PrimGrad<DIM, T> pl;
  primitiveGradient<DIM>(gr, s.u, s.ir, s.E * s.ir, ph, pl);
  const Comp<DIM, T>& lm = bc >= 3 ? b : l;
  T fl[NV], fb[NV];
  viscousNormalFlux<DIM>(pl, lm.u, lm.e * ph.inv_cv, n, ph, fl);
  PrimGrad<DIM, T> pb = pl;
  if (bc >= 4) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) pb.gT[k] = T(0.0);
  }
  viscousNormalFlux<DIM>(pb, b.u, b.e * ph.inv_cv, n, ph, fb);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    hv[v] = -0.5 * (fl[v] + fb[v]);
    h[v] = h[v] + hv[v];
  }
}

// Neighbour trace of the gradient pass at a boundary point (exchangeBoundaryPoint, generic): 2 U_b - U with
// U_b = U for farfield / inflow / outflow and the wall's boundary state otherwise.
template <int DIM, class T>
__device__ __forceinline__ void boundaryOtherOf(const T* ul, const T* gprim, const double* n, int bc, const Phys& ph,
                                                T* other) {
  constexpr int NV = DIM + 2;
  if (bc <= 2) {
#pragma unroll
    for (int v = 0; v < NV; ++v) other[v] = ul[v];
    return;
  }
  State<DIM, T> s;
  makeState<DIM>(s, ul, ph);
  Comp<DIM, T> l, g, b;
  compFromState<DIM>(s, l, ph);
  g.r = gprim[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gprim[1 + k];
  g.e = ph.cv * gprim[DIM + 1];
  g.p = ph.incomp ? weakPressure(g.r, ph) : ph.gm1 * g.r * g.e;
  boundaryState<DIM>(bc, n, l, g, ph, b);
  T ub[NV];
  ub[0] = b.r;
#pragma unroll
  for (int k = 0; k < DIM; ++k) ub[1 + k] = b.r * b.u[k];
  ub[DIM + 1] = energyOfComp<DIM>(b, ph);
#pragma unroll
  for (int v = 0; v < NV; ++v) other[v] = 2.0 * ub[v] - ul[v];
}

// Tangent of the boundary exchange: dother = (2 dU_b/dU - I) dU.
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) jvpExchangeBoundaryKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using D1 = Dual<1>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j;
  double n[DIM], gp[NV];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
  D1 ul[NV], gd[NV], o[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    ul[v].v = a.face[L + v * nfq]; ul[v].d[0] = a.dface[L + v * nfq];
    gd[v] = D1(gp[v]);
  }
  boundaryOtherOf<DIM>(ul, gd, n, bc, ph, o);
#pragma unroll
  for (int v = 0; v < NV; ++v) a.dother[L + v * nfq] = o[v].d[0];
}

// Transpose of the boundary exchange: lamTr += (2 dU_b/dU - I)^T lamUp; ghost += 2 (dU_b/dg)^T lamUp.
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) vjpExchangeBoundaryKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using DK = Dual<NV>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j;
  double n[DIM], gp[NV], lo[NV], ul[NV];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
#pragma unroll
  for (int v = 0; v < NV; ++v) { lo[v] = a.lamUp[L + v * nfq]; ul[v] = a.face[L + v * nfq]; }
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    DK x[NV], g[NV], o[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      x[v] = DK(ul[v]);
      g[v] = DK(gp[v]);
      if (side == 0) x[v].d[v] = 1.0; else g[v].d[v] = 1.0;
    }
    boundaryOtherOf<DIM>(x, g, n, bc, ph, o);
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double acc = 0.0;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc = fma(lo[v], o[v].d[w], acc);
      if (side == 0) a.lamTr[L + w * nfq] += acc;
      else if (a.lamGhost) a.lamGhost[t * NV + w] = fma(a.ghostScale, acc, a.lamGhost[t * NV + w]);
    }
  }
}

// Navier-Stokes boundary-face tangent: dH = |J_f| (dh/dU dU + dh/dG dG + dmu/mu hv).
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) jvpBoundaryNSKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using D1 = Dual<1>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j, LG = int64_t(sl) * NV * DIM * nfq + j;
  double n[DIM], gp[NV];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
  ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
  D1 ul[NV], gd[NV], gr[NV * DIM], h[NV], hv[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    ul[v].v = a.face[L + v * nfq]; ul[v].d[0] = a.dface[L + v * nfq];
    gd[v] = D1(gp[v]);
  }
#pragma unroll
  for (int c = 0; c < NV * DIM; ++c) { gr[c].v = a.faceGrad[LG + c * nfq]; gr[c].d[0] = a.dfaceGrad[LG + c * nfq]; }
  boundaryNSFluxOf<DIM>(ul, gr, gd, n, bc, ph, h, hv);
  const double mscale = ph.mu > 0.0 ? a.dmu / ph.mu : 0.0;
#pragma unroll
  for (int v = 0; v < NV; ++v) a.dflux[L + v * nfq] = fma(mscale, hv[v].v, h[v].d[0]) * area;
}

// Navier-Stokes boundary-face transpose: the trace (Dual<d+2>), gradient-trace (Dual<(d+2)d>) and ghost
// (Dual<d+2>) cotangents, and the viscosity term <lam_h, hv>.
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) vjpBoundaryNSKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2, NG = NV * DIM;
  using DK = Dual<NV>;
  using DG = Dual<NG>;
  __shared__ double sRed[kFaceThreads / 32];
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  double mupart = 0.0;
  if (f < a.nface) {
    const int j = int(t - f * nfq);
    const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
    const int64_t L = int64_t(sl) * NV * nfq + j, LG = int64_t(sl) * NV * DIM * nfq + j;
    double n[DIM], gp[NV], lh[NV], ul[NV], gg[NG];
#pragma unroll
    for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
    const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
    ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
#pragma unroll
    for (int v = 0; v < NV; ++v) { lh[v] = a.lamH[L + v * nfq] * area; ul[v] = a.face[L + v * nfq]; }
#pragma unroll
    for (int c = 0; c < NG; ++c) gg[c] = a.faceGrad[LG + c * nfq];
#pragma unroll
    for (int side = 0; side < 2; ++side) {  // 0: the trace, 1: the ghost primitive
      DK x[NV], g[NV], gr[NG], h[NV], hv[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        x[v] = DK(ul[v]);
        g[v] = DK(gp[v]);
        if (side == 0) x[v].d[v] = 1.0; else g[v].d[v] = 1.0;
      }
#pragma unroll
      for (int c = 0; c < NG; ++c) gr[c] = DK(gg[c]);
      boundaryNSFluxOf<DIM>(x, gr, g, n, bc, ph, h, hv);
      if (side == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) mupart = fma(lh[v], hv[v].v, mupart);
      }
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        double acc = 0.0;
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lh[v], h[v].d[w], acc);
        if (side == 0) a.lamTr[L + w * nfq] = acc;
        else if (a.lamGhost) a.lamGhost[t * NV + w] = fma(a.ghostScale, acc, a.lamGhost[t * NV + w]);
      }
    }
    {  // gradient traces
      DG x[NV], g[NV], gr[NG], h[NV], hv[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) { x[v] = DG(ul[v]); g[v] = DG(gp[v]); }
#pragma unroll
      for (int c = 0; c < NG; ++c) { gr[c] = DG(gg[c]); gr[c].d[c] = 1.0; }
      boundaryNSFluxOf<DIM>(x, gr, g, n, bc, ph, h, hv);
#pragma unroll
      for (int c = 0; c < NG; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lh[v], h[v].d[c], acc);
        a.lamTg[LG + c * nfq] = acc;
      }
    }
  }
  blockSum(mupart, a.muPart + blockIdx.x, sRed);
}

template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) jvpBoundaryKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using D1 = Dual<1>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j;
  double n[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
  double gp[NV];
  ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
  D1 ul[NV], gd[NV], h[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    ul[v].v = a.face[L + v * nfq]; ul[v].d[0] = a.dface[L + v * nfq];
    gd[v] = D1(gp[v]);
  }
  boundaryFluxOf<DIM>(ul, gd, n, bc, ph, h);
#pragma unroll
  for (int v = 0; v < NV; ++v) a.dflux[L + v * nfq] = h[v].d[0] * area;
}

template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) vjpBoundaryKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using DK = Dual<NV>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j;
  double n[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
  double lh[NV], ul[NV], gp[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) { lh[v] = a.lamH[L + v * nfq] * area; ul[v] = a.face[L + v * nfq]; }
  ghostPrimitiveOf<DIM>(a.ghost, t, ph, gp);
#pragma unroll
  for (int side = 0; side < 2; ++side) {  // 0: the interior trace, 1: the ghost primitive
    DK x[NV], g[NV], h[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      x[v] = DK(ul[v]);
      g[v] = DK(gp[v]);
      if (side == 0) x[v].d[v] = 1.0; else g[v].d[v] = 1.0;
    }
    boundaryFluxOf<DIM>(x, g, n, bc, ph, h);
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double acc = 0.0;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc = fma(lh[v], h[v].d[w], acc);
      if (side == 0) a.lamTr[L + w * nfq] = acc;
      else if (a.lamGhost) a.lamGhost[t * NV + w] = fma(a.ghostScale, acc, a.lamGhost[t * NV + w]);
    }
  }
}

// ---- tangent-linear --------------------------------------------------------------------------------------
// Face point: dH = |J_f| (dh/dUL dUL + dh/dUR dUR [+ dh/dG dG] + dmu/mu hv), scattered +/- as the forward.
template <int DIM, int FLUX, bool VISC>
__device__ __forceinline__ void jvpFacePoint(const AdjArgs& a, const Phys& ph, int64_t t) {
  constexpr int NV = DIM + 2;
  using D1 = Dual<1>;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
  D1 ul[NV], ur[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    ul[v].v = a.face[L + v * nfq]; ul[v].d[0] = a.dface[L + v * nfq];
    ur[v].v = a.face[R + v * nfq]; ur[v].d[0] = a.dface[R + v * nfq];
  }
  D1 gl[VISC ? NV * DIM : 1], gr[VISC ? NV * DIM : 1];
  if constexpr (VISC) {
    const int64_t LG = int64_t(sl) * NV * DIM * nfq + j, RG = int64_t(sr) * NV * DIM * nfq + jr;
#pragma unroll
    for (int c = 0; c < NV * DIM; ++c) {
      gl[c].v = a.faceGrad[LG + c * nfq]; gl[c].d[0] = a.dfaceGrad[LG + c * nfq];
      gr[c].v = a.faceGrad[RG + c * nfq]; gr[c].d[0] = a.dfaceGrad[RG + c * nfq];
    }
  }
  double n[DIM];
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
  const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
  D1 h[NV], hv[NV];
  faceFluxPoint<DIM, FLUX, VISC>(ul, ur, gl, gr, n, ph, h, hv);
  const double mscale = VISC && ph.mu > 0.0 ? a.dmu / ph.mu : 0.0;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = fma(mscale, hv[v].v, h[v].d[0]) * area;
    a.dflux[L + v * nfq] = x;
    a.dflux[R + v * nfq] = -x;
  }
}

template <int DIM, int FLUX, bool VISC>
__global__ void __launch_bounds__(kFaceThreads) jvpFaceKernel(AdjArgs a, Phys ph) {
  jvpFacePoint<DIM, FLUX, VISC>(a, ph, int64_t(blockIdx.x) * blockDim.x + threadIdx.x);
}

template <int DIM, int N>
struct AdjShape {
  using S = TensorShape<DIM, N>;
  static constexpr int NV = S::NV, NB = S::NB, NF = S::NF, NFQ = S::NFQ, USTRIDE = S::USTRIDE, FSTRIDE = S::FSTRIDE;
  static constexpr int GSTR = NV * DIM * NB;
  static constexpr int EPB = S::EPB;
  static constexpr int THREADS = S::THREADS;
  // tangent element tile: u, du | tangent flux slots | tangent contravariant fluxes [DIM][NV][NB]
  static constexpr size_t JVP_SMEM = size_t(EPB) * 8 * (2 * USTRIDE + FSTRIDE + DIM * NV * NB) + sizeof(TensorTables);
  // adjoint element tiles, each its own layout (the shared memory bounds how many CTAs an SM keeps):
  //   volume:   scaled cotangent s [NV][NB] | tables | one double per warp (the viscosity term's sum)
  //   gradient: t_b [DIM][NV][NB] (BR2: and v_b) | tables
  //   trace:    tables
  static constexpr size_t VOL_SMEM = size_t(EPB) * 8 * NV * NB + sizeof(TensorTables) + 8 * 32;
  static constexpr size_t GRAD_SMEM = size_t(EPB) * 8 * 2 * DIM * NV * NB + sizeof(TensorTables);  // also the bilinear form's s, w
  static constexpr size_t TRACE_SMEM = sizeof(TensorTables);
};

template <int DIM, int N>
__device__ __forceinline__ void loadTensorTables(TensorTables* T, const double* src) {
  double* dst = reinterpret_cast<double*>(T);
  for (int k = threadIdx.x; k < int(sizeof(TensorTables) / 8); k += blockDim.x) dst[k] = src[k];
}

// Tangent element kernel: dR = (1/|J|)[sum_b Dhat_b dQ_b - Lift dH]; RK combination of the tangents and
// the traces of the new tangent state (the forward stage kernel's structure on tangents).
template <int DIM, int N, bool VISC, bool AFF = true>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) jvpStageKernel(AdjArgs a, Phys ph) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB;
  using D1 = Dual<1>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE]
  double* sD = sU + EPB * A::USTRIDE;                // [EPB][USTRIDE] tangent state
  double* sF = sD + EPB * A::USTRIDE;                // [EPB][FSTRIDE] tangent flux slots
  double* sG = sF + EPB * A::FSTRIDE;                // [EPB][DIM][NV][NB] tangent fluxes
  TensorTables* T = reinterpret_cast<TensorTables*>(sG + EPB * DIM * NV * NB);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  for (int k = tid; k < ecount * A::USTRIDE; k += blockDim.x) {
    sU[k] = a.u[e0 * A::USTRIDE + k];
    sD[k] = a.du[e0 * A::USTRIDE + k];
  }
  for (int k = tid; k < ecount * A::FSTRIDE; k += blockDim.x) sF[k] = a.dflux[(a.faceBase + e0 * NF) * NV * NFQ + k];
  __syncthreads();
  double jinv = 0.0;
  if (active) {
    // affine: one metric per element; bilinear quadrangles: per node (the forward stage tile's geometry)
    const double* g = AFF ? a.geom + e * (DIM * DIM + 1) : a.geom + (e * NB + node) * (DIM * DIM + 1);
    double ja[DIM][DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
    jinv = g[DIM * DIM];
    D1 U[NV], gg[VISC ? NV * DIM : 1];
#pragma unroll
    for (int v = 0; v < NV; ++v) { U[v].v = sU[le * A::USTRIDE + v * NB + node]; U[v].d[0] = sD[le * A::USTRIDE + v * NB + node]; }
    if constexpr (VISC) {
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) {
        gg[c].v = a.grad[(e * NV * DIM + c) * NB + node];
        gg[c].d[0] = a.dgrad[(e * NV * DIM + c) * NB + node];
      }
    }
    D1 Q[DIM][NV], Qv[DIM][NV];
    nodeFlux<DIM, VISC>(U, gg, ja, ph, Q, Qv);
    const double mscale = VISC && ph.mu > 0.0 ? a.dmu / ph.mu : 0.0;
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) sG[((le * DIM + b) * NV + v) * NB + node] = fma(mscale, Qv[b][v].v, Q[b][v].d[0]);
  }
  __syncthreads();
  double dnew[NV];
  if (active) {
    double du[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) du[v] = 0.0;
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int ab = axisIndex<DIM, N>(node, b);
      const int base = node - ab * strideOf<DIM, N>(b);
      const double lm = T->liftm[ab], lp = T->liftp[ab];
      const int fm = T->axisFace[b][0], fp = T->axisFace[b][1];
      const int jm = T->nodeFacePoint[b][0][node], jp = T->nodeFacePoint[b][1][node];
      const double* G = sG + ((le * DIM + b) * NV) * NB + base;
      const double* Fm = sF + le * A::FSTRIDE + fm * NV * NFQ + jm;
      const double* Fp = sF + le * A::FSTRIDE + fp * NV * NFQ + jp;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double acc = du[v];
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(T->dhat[q][ab], G[v * NB + q * strideOf<DIM, N>(b)], acc);
        acc = fma(-lm, Fm[v * NFQ], acc);
        acc = fma(-lp, Fp[v * NFQ], acc);
        du[v] = acc;
      }
    }
    if (ph.source) {  // tangent of the buoyancy S |J| on the last momentum component
      D1 U[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) { U[v].v = sU[le * A::USTRIDE + v * NB + node]; U[v].d[0] = sD[le * A::USTRIDE + v * NB + node]; }
      State<DIM, D1> st;
      makeState<DIM>(st, U, ph);
      const D1 S = st.r * ph.beta * (temperatureOf(st, ph) - ph.tref);
      du[DIM] = fma(S.d[0], 1.0 / jinv, du[DIM]);
    }
    const int64_t gi = e * A::USTRIDE + node;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      if (a.drate) a.drate[gi + v * NB] = du[v] * jinv;
      dnew[v] = fma(a.c2dt * jinv, du[v], fma(a.c1, sD[le * A::USTRIDE + v * NB + node], a.c0 * (a.dbase ? a.dbase[gi + v * NB] : 0.0)));
    }
  }
  __syncthreads();
  if (!a.dout) return;
  if (active) {
    const int64_t gi = e * A::USTRIDE + node;
#pragma unroll
    for (int v = 0; v < NV; ++v) { a.dout[gi + v * NB] = dnew[v]; sD[le * A::USTRIDE + v * NB + node] = dnew[v]; }
  }
  __syncthreads();
  if (!a.dtrace) return;
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f];
    const double* coef = T->faceEnd[f] ? T->endp : T->endm;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const double* u = sD + te * A::USTRIDE + base;
    double* out = a.dtrace + (a.faceBase + (e0 + te) * NF + f) * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < N; ++q) acc = fma(coef[q], u[v * NB + q * st], acc);
      out[v * NFQ] = acc;
    }
  }
}

// ---- adjoint -----------------------------------------------------------------------------------------
// Deterministic per-CTA sum of one value per thread into part[blockIdx.x].
__device__ __forceinline__ void blockSum(double x, double* part, double* sRed) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
  const int warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) sRed[warp] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nwarp; ++w) s += sRed[w];
    *part = s;
  }
}

// V1: s = lam/|J|; lamQ_b by the transposed derivative; node Jacobians by Dual<NV> over U;
// lamG (NS) by the viscous transpose; lamH by the transposed lift.  muPart[tile] = <lamQ, Qv>.
template <int DIM, int N, bool VISC, bool GEN, bool AFF = true>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpVolumeKernel(AdjArgs a, Phys ph) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sS = reinterpret_cast<double*>(smem_raw);  // [EPB][NV][NB] s = lam / |J|
  TensorTables* T = reinterpret_cast<TensorTables*>(sS + EPB * NV * NB);
  double* sRed = reinterpret_cast<double*>(T + 1);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  double jinv = 0.0;
  const double* geo = AFF ? a.geom + e * (DIM * DIM + 1) : a.geom + (e * NB + node) * (DIM * DIM + 1);
  if (active) {
    jinv = geo[DIM * DIM];
#pragma unroll
    for (int v = 0; v < NV; ++v) sS[(le * NV + v) * NB + node] = jinv * a.lam[e * A::USTRIDE + v * NB + node];
  }
  __syncthreads();
  double mupart = 0.0;
  if (active) {
    const double* g = geo;
    double ja[DIM][DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
    // lamQ_b at this node: sum over the line of dhat[q=this][a] s(a)
    double lq[DIM][NV];
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int ab = axisIndex<DIM, N>(node, b);
      const int st = strideOf<DIM, N>(b);
      const int base = node - ab * st;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(T->dhat[ab][q], sS[(le * NV + v) * NB + base + q * st], acc);
        lq[b][v] = acc;
      }
    }
    // Jacobian transposes with respect to U (G held fixed) and, for Navier-Stokes, G
    double Uv[NV], lu[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) Uv[v] = a.u[e * A::USTRIDE + v * NB + node];
    if constexpr (GEN) {  // the dual-number transpose (incompressible model, buoyancy)
      double gg[VISC ? NV * DIM : 1], lg[VISC ? NV * DIM : 1];
      if constexpr (VISC) {
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) gg[c] = a.grad[(e * NV * DIM + c) * NB + node];
      }
      mupart = volumeReverseGeneric<DIM, VISC>(Uv, gg, ja, lq, a.lam[e * A::USTRIDE + DIM * NB + node], ph, lu, lg);
      if constexpr (VISC) {
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) a.lamG[(e * NV * DIM + c) * NB + node] = lg[c];
      }
    } else {
    eulerVolumeReverse<DIM>(Uv, ja, lq, ph, lu);
    if constexpr (VISC) {
      // lamF[c][v] = cotangent of Fv_c(v): Q_b contains -sum_c ja[b][c] Fv_c
      double lamF[DIM][NV], gg[NV * DIM], lg[NV * DIM];
#pragma unroll
      for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double acc = 0.0;
#pragma unroll
          for (int b = 0; b < DIM; ++b) acc = fma(-ja[b][c], lq[b][v], acc);
          lamF[c][v] = acc;
        }
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) { gg[c] = a.grad[(e * NV * DIM + c) * NB + node]; lg[c] = 0.0; }
      mupart = viscousReverse<DIM>(Uv, gg, lamF, ph, lu, lg);
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) a.lamG[(e * NV * DIM + c) * NB + node] = lg[c];
    }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) a.lamU[e * A::USTRIDE + v * NB + node] = lu[v];
  }
  if constexpr (VISC) blockSum(mupart, a.muPart + blockIdx.x, sRed);
  // transposed lift: lamH(f, j) = -sum over the line through (f, j) of lift(a) s(a)
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f];
    const double* lift = T->faceEnd[f] ? T->liftp : T->liftm;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const double* s = sS + te * NV * NB + base;
    double* out = a.lamH + (a.faceBase + (e0 + te) * NF + f) * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < N; ++q) acc = fma(-lift[q], s[v * NB + q * st], acc);
      out[v * NFQ] = acc;
    }
  }
}

// V2: face point.  lam_h = lamH(L) - lamH(R) (the +/- scatter); trace cotangents of the convective flux
// (Roe: hand-written reverse sweep; other fluxes: Dual<NV> passes seeded on UL and on UR) and, for
// Navier-Stokes, of each side's viscous flux (state and gradient parts); muPart = <lam_h, hv>.
template <int DIM, int FLUX, bool VISC, bool GEN>
__global__ void __launch_bounds__(kFaceThreads) vjpFaceKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using DK = Dual<NV>;
  __shared__ double sRed[kFaceThreads / 32];
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  double mupart = 0.0;
  if (f < a.nface) {
    const int j = int(t - f * nfq);
    const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
    const int jr = pairedPoint<DIM>(a, j, rot, nfq);
    const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
    double n[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) n[k] = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[k];
    const double area = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq)[3];
    double lh[NV], ul[NV], ur[NV], laml[NV], lamr[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      lh[v] = (a.lamH[L + v * nfq] - a.lamH[R + v * nfq]) * area;
      ul[v] = a.face[L + v * nfq];
      ur[v] = a.face[R + v * nfq];
      laml[v] = 0.0;
      lamr[v] = 0.0;
    }
    if constexpr (FLUX == 3) {
      roeReverse<DIM>(ul, ur, n, ph, lh, laml, lamr);
    } else {
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        DK xl[NV], xr[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          xl[v] = DK(ul[v]);
          xr[v] = DK(ur[v]);
          if (side == 0) xl[v].d[v] = 1.0; else xr[v].d[v] = 1.0;
        }
        State<DIM, DK> l, r;
        makeState<DIM>(l, xl, ph);
        makeState<DIM>(r, xr, ph);
        DK h[NV];
        convectiveFlux<DIM, FLUX>(l, r, n, ph, h);
        double* out = side == 0 ? laml : lamr;
#pragma unroll
        for (int w = 0; w < NV; ++w) {
          double acc = 0.0;
#pragma unroll
          for (int v = 0; v < NV; ++v) acc = fma(lh[v], h[v].d[w], acc);
          out[w] = acc;
        }
      }
    }
    if constexpr (VISC) {
      // h contains -1/2 Fv(U_side, G_side).n on each side: lamF[c][v] = -1/2 n_c lam_h(v)
      const int64_t LG = int64_t(sl) * NV * DIM * nfq + j, RG = int64_t(sr) * NV * DIM * nfq + jr;
      double lamF[DIM][NV];
#pragma unroll
      for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int v = 0; v < NV; ++v) lamF[c][v] = -0.5 * n[c] * lh[v];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        const int64_t G0 = side == 0 ? LG : RG;
        double gg[NV * DIM], lg[NV * DIM];
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) { gg[c] = a.faceGrad[G0 + c * nfq]; lg[c] = 0.0; }
        if constexpr (GEN)
          mupart += faceViscousReverseGeneric<DIM>(side == 0 ? ul : ur, gg, n, lh, ph, side == 0 ? laml : lamr, lg);
        else
          mupart += viscousReverse<DIM>(side == 0 ? ul : ur, gg, lamF, ph, side == 0 ? laml : lamr, lg);
        double* out = a.lamTg + G0;
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) out[c * nfq] = lg[c];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      a.lamTr[L + v * nfq] = laml[v];
      a.lamTr[R + v * nfq] = lamr[v];
    }
  }
  if constexpr (VISC) blockSum(mupart, a.muPart + blockIdx.x, sRed);
}

// V3 (NS): lamG_total = lamG + T^T lamTg; t_b = (1/|J|) sum_k JA[b][k] lamG_total(k); lamU -= Dhat_b^T t_b;
// lamUp(face of axis b, end) = +-sum over the line of lift(a) t_b(a).
template <int DIM, int N>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpGradientKernel(AdjArgs a) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB, GS = NV * DIM;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sT = reinterpret_cast<double*>(smem_raw);  // [EPB][DIM][NV][NB]  t_b
  TensorTables* T = reinterpret_cast<TensorTables*>(sT + EPB * DIM * NV * NB);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  __syncthreads();
  if (active) {
    const double* g = a.geom + e * (DIM * DIM + 1);
    double ja[DIM][DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
    const double jinv = g[DIM * DIM];
    double lg[GS];
#pragma unroll
    for (int c = 0; c < GS; ++c) lg[c] = a.lamG[(e * GS + c) * NB + node];
    // transposed gradient traces: the node is on one line per axis, with a face point at each end
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int ab = axisIndex<DIM, N>(node, b);
#pragma unroll
      for (int en = 0; en < 2; ++en) {
        const int f = T->axisFace[b][en];
        const int j = T->nodeFacePoint[b][en][node];
        const double c = en ? T->endp[ab] : T->endm[ab];
        const double* src = a.lamTg + (a.faceBase + e * NF + f) * GS * NFQ + j;
#pragma unroll
        for (int k = 0; k < GS; ++k) lg[k] = fma(c, src[k * NFQ], lg[k]);
      }
    }
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) acc = fma(ja[b][k], lg[v * DIM + k], acc);
        sT[((le * DIM + b) * NV + v) * NB + node] = jinv * acc;
      }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const int ab = axisIndex<DIM, N>(node, b);
        const int st = strideOf<DIM, N>(b);
        const int base = node - ab * st;
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(T->dhat[ab][q], sT[((le * DIM + b) * NV + v) * NB + base + q * st], acc);
      }
      a.lamU[e * A::USTRIDE + v * NB + node] -= acc;
    }
  }
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f], en = T->faceEnd[f];
    const double* lift = en ? T->liftp : T->liftm;
    const double sign = en ? 1.0 : -1.0;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const double* tb = sT + (te * DIM + axis) * NV * NB + base;
    double* out = a.lamUp + (a.faceBase + (e0 + te) * NF + f) * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < N; ++q) acc = fma(lift[q], tb[v * NB + q * st], acc);
      out[v * NFQ] = sign * acc;
    }
  }
}

// V3 for BR2.  The node gradient (volume terms) is the BR1 gradient G = (1/|J|) sum_b JA_b (lift_b U+ - Dhat_b U);
// the gradient trace at face f is the trace of the volume part V = (1/|J|) sum_b JA_b (lift_b {U} - Dhat_b U)
// plus face f's own lift, cl nF_f 1/2 (U+ - U-) at the point (tensorGradientTile, BR2).  With
// t_b = (1/|J|) sum_k JA[b][k] lamG(k) and v_b the same of T^T lamTg:
//   lamU  -= Dhat_b^T (t_b + v_b)
//   lamUp  = +-lift (t_b + v_b/2) + cl/2 nF.lamTg         (the neighbour traces U+)
//   lamTr += +-lift v_b/2         - cl/2 nF.lamTg         (the own traces U-)
template <int DIM, int N>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpGradientBR2Kernel(AdjArgs a) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB, GS = NV * DIM;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sT = reinterpret_cast<double*>(smem_raw);  // [EPB][DIM][NV][NB]  t_b + v_b
  double* sV = sT + EPB * DIM * NV * NB;             // [EPB][DIM][NV][NB]  v_b
  TensorTables* T = reinterpret_cast<TensorTables*>(sV + EPB * DIM * NV * NB);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  __syncthreads();
  if (active) {
    const double* g = a.geom + e * (DIM * DIM + 1);
    double ja[DIM][DIM];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
    const double jinv = g[DIM * DIM];
    double lg[GS], lv[GS];
#pragma unroll
    for (int c = 0; c < GS; ++c) { lg[c] = a.lamG[(e * GS + c) * NB + node]; lv[c] = 0.0; }
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int ab = axisIndex<DIM, N>(node, b);
#pragma unroll
      for (int en = 0; en < 2; ++en) {
        const int f = T->axisFace[b][en];
        const int j = T->nodeFacePoint[b][en][node];
        const double c = en ? T->endp[ab] : T->endm[ab];
        const double* src = a.lamTg + (a.faceBase + e * NF + f) * GS * NFQ + j;
#pragma unroll
        for (int k = 0; k < GS; ++k) lv[k] = fma(c, src[k * NFQ], lv[k]);
      }
    }
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double at = 0.0, av = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) { at = fma(ja[b][k], lg[v * DIM + k], at); av = fma(ja[b][k], lv[v * DIM + k], av); }
        sT[((le * DIM + b) * NV + v) * NB + node] = jinv * (at + av);
        sV[((le * DIM + b) * NV + v) * NB + node] = jinv * av;
      }
  }
  __syncthreads();
  if (active) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const int ab = axisIndex<DIM, N>(node, b);
        const int st = strideOf<DIM, N>(b);
        const int base = node - ab * st;
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(T->dhat[ab][q], sT[((le * DIM + b) * NV + v) * NB + base + q * st], acc);
      }
      a.lamU[e * A::USTRIDE + v * NB + node] -= acc;
    }
  }
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f], en = T->faceEnd[f];
    const double* lift = en ? T->liftp : T->liftm;
    const double* coef = en ? T->endp : T->endm;
    const double sign = en ? 1.0 : -1.0;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const int64_t ee = e0 + te;
    const double* gm = a.geom + ee * (DIM * DIM + 1);
    double cl = 0.0;  // lift trace factor sum_q l_q(end) lift_q / |J| (affine)
#pragma unroll
    for (int q = 0; q < N; ++q) cl = fma(coef[q], lift[q], cl);
    cl *= gm[DIM * DIM];
    const double* tb = sT + (te * DIM + axis) * NV * NB + base;
    const double* vb = sV + (te * DIM + axis) * NV * NB + base;
    const int64_t slot = a.faceBase + ee * NF + f;
    const double* ltg = a.lamTg + slot * GS * NFQ + j;
    double* up = a.lamUp + slot * NV * NFQ + j;
    double* tr = a.lamTr + slot * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double at = 0.0, av = 0.0, nl = 0.0;
#pragma unroll
      for (int q = 0; q < N; ++q) { at = fma(lift[q], tb[v * NB + q * st], at); av = fma(lift[q], vb[v * NB + q * st], av); }
#pragma unroll
      for (int k = 0; k < DIM; ++k) nl = fma(sign * gm[axis * DIM + k], ltg[(v * DIM + k) * NFQ], nl);
      up[v * NFQ] = fma(0.5 * cl, nl, sign * fma(-0.5, av, at));
      tr[v * NFQ] += fma(-0.5 * cl, nl, 0.5 * sign * av);
    }
  }
}

// V3 for non-affine tensor blocks -- bilinear and curved quadrangles, trilinear and curved hexahedra -- (per-node
// metric ja_q and 1/|J|_q, n|J_f| from the face metric per face or per face point; tensorGradientTile's
// non-affine form).  Forward, at node m along each axis b:
//   tot_k(m) = sum_b [ lift(+) nF(b,+)_k U+(b,+) + lift(-) nF(b,-)_k U+(b,-) - sum_q Dhat[q][m] U_q ja_q[b][k] ]
//   grad = tot / |J|_m (BR1 gradient traces: its traces); BR2: vol from {U} in place of U+, gradient trace at
//   (f, j) = trace(vol / |J|) + cl nF_f . (U+ - U-)/2 with cl = sum_q end_q lift_q / |J|_q.
// Transposed, with s = (1/|J|) (lamG + [BR1] T^T lamTg), w = (1/|J|) T^T lamTg (BR2):
//   lamU_q -= sum_b sum_k ja_q[b][k] (Dhat^T (s + w)_k)_q,
//   lamUp(f, j) = sum_line lift nF_f . s  [+ BR2: (1/2) sum_line lift nF_f . w + (cl/2) nF_f . lamTg(f, j)],
//   BR2: lamTr(f, j) += (1/2) sum_line lift nF_f . w - (cl/2) nF_f . lamTg(f, j).
template <int DIM, int N, bool BR2>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpGradientBilinearKernel(AdjArgs a) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB, GS = NV * DIM, GSZ = DIM * DIM + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sS = reinterpret_cast<double*>(smem_raw);  // [EPB][GS][NB]  s
  double* sW = sS + EPB * GS * NB;                   // [EPB][GS][NB]  w (BR2)
  TensorTables* T = reinterpret_cast<TensorTables*>(sW + EPB * GS * NB);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  __syncthreads();
  if (active) {
    const double jinv = a.geom[(e * NB + node) * GSZ + DIM * DIM];
    double lg[GS], lv[GS];
#pragma unroll
    for (int c = 0; c < GS; ++c) { lg[c] = a.lamG[(e * GS + c) * NB + node]; lv[c] = 0.0; }
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int ab = axisIndex<DIM, N>(node, b);
#pragma unroll
      for (int en = 0; en < 2; ++en) {
        const int f = T->axisFace[b][en];
        const int j = T->nodeFacePoint[b][en][node];
        const double c = en ? T->endp[ab] : T->endm[ab];
        const double* src = a.lamTg + (a.faceBase + e * NF + f) * GS * NFQ + j;
#pragma unroll
        for (int k = 0; k < GS; ++k) lv[k] = fma(c, src[k * NFQ], lv[k]);
      }
    }
#pragma unroll
    for (int c = 0; c < GS; ++c) {
      sS[(le * GS + c) * NB + node] = jinv * (BR2 ? lg[c] : lg[c] + lv[c]);
      sW[(le * GS + c) * NB + node] = BR2 ? jinv * lv[c] : 0.0;
    }
  }
  __syncthreads();
  if (active) {
    const double* g = a.geom + (e * NB + node) * GSZ;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const int ab = axisIndex<DIM, N>(node, b);
        const int st = strideOf<DIM, N>(b);
        const int base = node - ab * st;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double d = 0.0;
#pragma unroll
          for (int q = 0; q < N; ++q) {
            const int o = (le * GS + v * DIM + k) * NB + base + q * st;
            d = fma(T->dhat[ab][q], sS[o] + sW[o], d);
          }
          acc = fma(g[b * DIM + k], d, acc);
        }
      }
      a.lamU[e * A::USTRIDE + v * NB + node] -= acc;
    }
  }
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f], en = T->faceEnd[f];
    const double* lift = en ? T->liftp : T->liftm;
    const double* coef = en ? T->endp : T->endm;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const int64_t ee = e0 + te;
    const double* nF = a.fmetric + (a.fmetricPoint ? (ee * NF + f) * NFQ + j : ee * NF + f) * DIM;
    double cl = 0.0;
    if constexpr (BR2) {
#pragma unroll
      for (int q = 0; q < N; ++q) cl = fma(coef[q] * lift[q], a.geom[(ee * NB + base + q * st) * GSZ + DIM * DIM], cl);
    }
    const int64_t slot = a.faceBase + ee * NF + f;
    const double* ltg = a.lamTg + slot * GS * NFQ + j;
    double* up = a.lamUp + slot * NV * NFQ + j;
    double* tr = a.lamTr + slot * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double at = 0.0, av = 0.0, nl = 0.0;
#pragma unroll
      for (int q = 0; q < N; ++q) {
        double ns = 0.0, nw = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          const int o = (te * GS + v * DIM + k) * NB + base + q * st;
          ns = fma(nF[k], sS[o], ns);
          nw = fma(nF[k], sW[o], nw);
        }
        at = fma(lift[q], ns, at);
        av = fma(lift[q], nw, av);
      }
      if constexpr (BR2) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) nl = fma(nF[k], ltg[(v * DIM + k) * NFQ], nl);
        up[v * NFQ] = fma(0.5 * cl, nl, fma(0.5, av, at));
        tr[v * NFQ] += fma(-0.5 * cl, nl, 0.5 * av);
      } else {
        up[v * NFQ] = at;
      }
    }
  }
}

// V4 (NS): transposed exchange, lamTr(R, jr) += lamUp(L, j) and lamTr(L, j) += lamUp(R, jr).
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) vjpExchangeKernel(AdjArgs a) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = a.lamUp[L + v * nfq], y = a.lamUp[R + v * nfq];
    a.lamTr[R + v * nfq] += x;
    a.lamTr[L + v * nfq] += y;
  }
}

// V5: lamU += T^T lamTr, then the RK combination of the stage's cotangents.
template <int DIM, int N>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpTraceKernel(AdjArgs a) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TensorTables* T = reinterpret_cast<TensorTables*>(smem_raw);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  const int le = tid / NB, node = tid - le * NB;
  const int64_t e = e0 + le;
  loadTensorTables<DIM, N>(T, a.tables);
  __syncthreads();
  if (le >= ecount) return;
  double lu[NV];
  const int64_t gi = e * A::USTRIDE + node;
#pragma unroll
  for (int v = 0; v < NV; ++v) lu[v] = a.lamU[gi + v * NB];
#pragma unroll
  for (int b = 0; b < DIM; ++b) {
    const int ab = axisIndex<DIM, N>(node, b);
#pragma unroll
    for (int en = 0; en < 2; ++en) {
      const int f = T->axisFace[b][en];
      const int j = T->nodeFacePoint[b][en][node];
      const double c = en ? T->endp[ab] : T->endm[ab];
      const double* src = a.lamTr + (a.faceBase + e * NF + f) * NV * NFQ + j;
#pragma unroll
      for (int v = 0; v < NV; ++v) lu[v] = fma(c, src[v * NFQ], lu[v]);
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double li = a.lamIn ? a.lamIn[gi + v * NB] : 0.0;
    if (a.accumulateAll) {
      a.lamBase[gi + v * NB] += fma(a.c2dt, lu[v], (a.c0 + a.c1) * li);
    } else {
      if (a.lamStage) a.lamStage[gi + v * NB] = fma(a.c2dt, lu[v], a.c1 * li);
      if (a.lamBase) a.lamBase[gi + v * NB] += a.c0 * li;
      if (!a.lamStage && !a.lamBase) a.lamU[gi + v * NB] = lu[v];
    }
  }
}

}  // namespace sdg
