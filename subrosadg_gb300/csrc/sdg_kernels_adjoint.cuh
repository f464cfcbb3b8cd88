// Tangent-linear (JVP) and adjoint (VJP) kernels of the residual of affine tensor blocks (quadrangles
// P>=2 and hexahedra), Euler or Navier-Stokes BR1, interior faces.
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
  const T ep = s.E + s.p;
  T tau[DIM][DIM], q[DIM];
  if constexpr (VISC) {
    PrimGrad<DIM, T> pg;
    primitiveGradient<DIM>(g, s.u, s.ir, s.E * s.ir, ph, pg);
    T u2 = T(0.0);
#pragma unroll
    for (int k = 0; k < DIM; ++k) u2 = fmaT(s.u[k], s.u[k], u2);
    viscousTensor<DIM>(pg, s.u, fmaT(-0.5, u2, s.E * s.ir) * ph.inv_cv, ph, tau, q);
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
      viscousNormalFlux<DIM>(pg, l.u, fmaT(-0.5, u2, l.E * l.ir) * ph.inv_cv, n, ph, fl);
    }
    {
      PrimGrad<DIM, T> pg;
      primitiveGradient<DIM>(gr, r.u, r.ir, r.E * r.ir, ph, pg);
      T u2 = T(0.0);
#pragma unroll
      for (int k = 0; k < DIM; ++k) u2 = fmaT(r.u[k], r.u[k], u2);
      viscousNormalFlux<DIM>(pg, r.u, fmaT(-0.5, u2, r.E * r.ir) * ph.inv_cv, n, ph, fr);
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
  int n1d, epb;
};

// ---- tangent-linear --------------------------------------------------------------------------------------
// Face point: dH = |J_f| (dh/dUL dUL + dh/dUR dUR [+ dh/dG dG] + dmu/mu hv), scattered +/- as the forward.
template <int DIM, int FLUX, bool VISC>
__device__ __forceinline__ void jvpFacePoint(const AdjArgs& a, const Phys& ph, int64_t t) {
  constexpr int NV = DIM + 2;
  using D1 = Dual<1>;
  const int n1d = a.n1d;
  const int nfq = DIM == 2 ? n1d : n1d * n1d;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = rightPoint<DIM>(j, rot, n1d);
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
  for (int k = 0; k < DIM; ++k) n[k] = a.fgeo[f * 4 + k];
  const double area = a.fgeo[f * 4 + 3];
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
  // adjoint element tiles: scaled cotangent s [NV][NB] | node-gradient cotangent [NV*DIM][NB] |
  // t_b [DIM][NV][NB] | slot cotangents (FSTRIDE * DIM for the gradient traces)
  static constexpr size_t VJP_SMEM =
      size_t(EPB) * 8 * (USTRIDE + GSTR + DIM * NV * NB + FSTRIDE * DIM) + sizeof(TensorTables);
};

template <int DIM, int N>
__device__ __forceinline__ void loadTensorTables(TensorTables* T, const double* src) {
  double* dst = reinterpret_cast<double*>(T);
  for (int k = threadIdx.x; k < int(sizeof(TensorTables) / 8); k += blockDim.x) dst[k] = src[k];
}

// Tangent element kernel: dR = (1/|J|)[sum_b Dhat_b dQ_b - Lift dH]; RK combination of the tangents and
// the traces of the new tangent state (the forward stage kernel's structure on tangents).
template <int DIM, int N, bool VISC>
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
    const double* g = a.geom + e * (DIM * DIM + 1);
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
template <int DIM, int N, bool VISC>
__global__ void __launch_bounds__(TensorShape<DIM, N>::THREADS) vjpVolumeKernel(AdjArgs a, Phys ph) {
  using A = AdjShape<DIM, N>;
  constexpr int NV = A::NV, NB = A::NB, NF = A::NF, NFQ = A::NFQ, EPB = A::EPB;
  using DK = Dual<NV>;
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
  if (active) {
    jinv = a.geom[e * (DIM * DIM + 1) + DIM * DIM];
#pragma unroll
    for (int v = 0; v < NV; ++v) sS[(le * NV + v) * NB + node] = jinv * a.lam[e * A::USTRIDE + v * NB + node];
  }
  __syncthreads();
  double mupart = 0.0;
  if (active) {
    const double* g = a.geom + e * (DIM * DIM + 1);
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
    // Jacobian with respect to U (G held fixed): one Dual<NV> pass
    DK U[NV], gg[VISC ? NV * DIM : 1];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      U[v] = DK(a.u[e * A::USTRIDE + v * NB + node]);
      U[v].d[v] = 1.0;
    }
    if constexpr (VISC) {
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) gg[c] = DK(a.grad[(e * NV * DIM + c) * NB + node]);
    }
    DK Q[DIM][NV], Qv[DIM][NV];
    nodeFlux<DIM, VISC>(U, gg, ja, ph, Q, Qv);
#pragma unroll
    for (int w = 0; w < NV; ++w) {
      double acc = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lq[b][v], Q[b][v].d[w], acc);
      a.lamU[e * A::USTRIDE + w * NB + node] = acc;
    }
    if constexpr (VISC) {
#pragma unroll
      for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int v = 0; v < NV; ++v) mupart = fma(lq[b][v], Qv[b][v].v, mupart);
      // lamF[c][v] = lambda of Fv_c(v): Q_b contains -sum_c ja[b][c] Fv_c
      double lamF[DIM][NV];
#pragma unroll
      for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double acc = 0.0;
#pragma unroll
          for (int b = 0; b < DIM; ++b) acc = fma(-ja[b][c], lq[b][v], acc);
          lamF[c][v] = acc;
        }
      double Uv[NV], lg[NV * DIM];
#pragma unroll
      for (int v = 0; v < NV; ++v) Uv[v] = U[v].v;
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) lg[c] = 0.0;
      viscousTransposeG<DIM>(Uv, ph, lamF, lg);
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) a.lamG[(e * NV * DIM + c) * NB + node] = lg[c];
    }
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

// V2: face point.  lam_h = lamH(L) - lamH(R) (the +/- scatter); trace cotangents from Dual<NV> passes
// seeded on UL and on UR; NS gradient-trace cotangents by the viscous transpose; muPart = <lam_h, hv>.
template <int DIM, int FLUX, bool VISC>
__global__ void __launch_bounds__(kFaceThreads) vjpFaceKernel(AdjArgs a, Phys ph) {
  constexpr int NV = DIM + 2;
  using DK = Dual<NV>;
  __shared__ double sRed[kFaceThreads / 32];
  const int n1d = a.n1d;
  const int nfq = DIM == 2 ? n1d : n1d * n1d;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  double mupart = 0.0;
  if (f < a.nface) {
    const int j = int(t - f * nfq);
    const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
    const int jr = rightPoint<DIM>(j, rot, n1d);
    const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
    const int64_t LG = int64_t(sl) * NV * DIM * nfq + j, RG = int64_t(sr) * NV * DIM * nfq + jr;
    double n[DIM];
#pragma unroll
    for (int k = 0; k < DIM; ++k) n[k] = a.fgeo[f * 4 + k];
    const double area = a.fgeo[f * 4 + 3];
    double lh[NV], ul[NV], ur[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      lh[v] = (a.lamH[L + v * nfq] - a.lamH[R + v * nfq]) * area;
      ul[v] = a.face[L + v * nfq];
      ur[v] = a.face[R + v * nfq];
    }
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      DK xl[NV], xr[NV], gl[VISC ? NV * DIM : 1], gr[VISC ? NV * DIM : 1];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        xl[v] = DK(ul[v]);
        xr[v] = DK(ur[v]);
        if (side == 0) xl[v].d[v] = 1.0; else xr[v].d[v] = 1.0;
      }
      if constexpr (VISC) {
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) { gl[c] = DK(a.faceGrad[LG + c * nfq]); gr[c] = DK(a.faceGrad[RG + c * nfq]); }
      }
      DK h[NV], hv[NV];
      faceFluxPoint<DIM, FLUX, VISC>(xl, xr, gl, gr, n, ph, h, hv);
      if (side == 0 && VISC) {
#pragma unroll
        for (int v = 0; v < NV; ++v) mupart = fma(lh[v], hv[v].v, mupart);
      }
      double* out = a.lamTr + (side == 0 ? L : R);
#pragma unroll
      for (int w = 0; w < NV; ++w) {
        double acc = 0.0;
#pragma unroll
        for (int v = 0; v < NV; ++v) acc = fma(lh[v], h[v].d[w], acc);
        out[w * nfq] = acc;
      }
    }
    if constexpr (VISC) {
      // h contains -1/2 Fv(U_side, G_side).n on each side: lamF[c][v] = -1/2 n_c lam_h(v)
      double lamF[DIM][NV];
#pragma unroll
      for (int c = 0; c < DIM; ++c)
#pragma unroll
        for (int v = 0; v < NV; ++v) lamF[c][v] = -0.5 * n[c] * lh[v];
#pragma unroll
      for (int side = 0; side < 2; ++side) {
        double lg[NV * DIM];
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) lg[c] = 0.0;
        viscousTransposeG<DIM>(side == 0 ? ul : ur, ph, lamF, lg);
        double* out = a.lamTg + (side == 0 ? LG : RG);
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) out[c * nfq] = lg[c];
      }
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

// V4 (NS): transposed exchange, lamTr(R, jr) += lamUp(L, j) and lamTr(L, j) += lamUp(R, jr).
template <int DIM>
__global__ void __launch_bounds__(kFaceThreads) vjpExchangeKernel(AdjArgs a) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = DIM == 2 ? n1d : n1d * n1d;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = rightPoint<DIM>(j, rot, n1d);
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
