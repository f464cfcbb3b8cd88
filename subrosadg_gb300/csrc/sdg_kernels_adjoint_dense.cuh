// Tangent-linear (JVP) and adjoint (VJP) element kernels of dense (modal) blocks -- triangles and first-order
// quadrangles -- for the Euler equations (compressible or incompressible, with the Boussinesq source; affine or
// bilinear elements) and for Navier-Stokes BR1 / BR2 (affine elements).  The face kernels of
// sdg_kernels_adjoint.cuh serve these blocks unchanged: they work on the face slots, whose layout
// [slot][nv][nfq] (gradient traces [slot][nv*2][nfq]) is the same for every block kind.
//
// Forward residual of a dense block (denseStageTile, SpatialDiscrete.cpp:194-266,1016-1032):
//   U_q = Phi U                           values at the volume points        (linear)
//   Q_b(U_q) = F(U_q) . |J| dxi_b/dx      contravariant fluxes               (pointwise, nonlinear)
//   R = sum_{q,b} Q_b dPhiw_b - sum_fj F_fj Phifw_fj (+ sum_q w_q |J| S(U_q) Phi on the last momentum)
//   du = s M^-1 R                         s = 1/|J| with M_ref^-1 (affine), s = 1 with the element's M^-1
//   traces Tr = Phi_f U                   (linear)
// The tangent applies the linear maps to tangents and the pointwise maps through Dual<1>; the adjoint is the
// transposed sequence:
//   lamR = s M^-T lam;  lamQ_b(q) = dPhiw_b lamR;  lamH(fj) = -Phifw_fj lamR (the flux slots)
//   lamU_q = sum_b (dQ_b/dU)^T lamQ_b (+ lamS dS/dU),  lamU = Phi^T lamU_q;   then lamU += Phi_f^T lamTr.
// Navier-Stokes adds the viscous fluxes of the modal gradient w at the points (Q_b depends on U_q and
// G_q = Phi w: lamw = Phi^T lamG_q) and the transposed gradient pass (vjpDenseGradientKernel).
#pragma once
#include "sdg_kernels_adjoint.cuh"
#include "sdg_kernels_dense.cuh"

namespace sdg {

template <int NB, int NQ, int NFQ, int NF, int DIM = 2>
struct DenseAdjShape {
  static constexpr int NV = DIM + 2, NFP = NF * NFQ;
  static constexpr int USTRIDE = (NV * NB + 1) & ~1;
  static constexpr int FSTRIDE = NF * NV * NFQ;
  static constexpr int EPB = 8, THREADS = 256;
  // phi | dphiw | phif | phifw | mref (the forward dense tables' leading part) | phiw (volume source weights)
  static constexpr int TABLES = NQ * NB * (1 + DIM) + NFP * NB * 2 + NB * NB;
  static constexpr int PHIW = TABLES + DIM * NB * NB + NF * NB * NFQ + NF * NFQ * NFQ;
  // tangent: u, du | tangent flux slots | tangent fluxes [d][NV][NQ] | tangent source [NQ] | tangent residual
  static constexpr int JVP_PER = 2 * USTRIDE + FSTRIDE + DIM * NV * NQ + NQ + NV * NB;
  // adjoint: lamR [NV][NB] | point cotangents [NV][NQ] | Navier-Stokes: point gradient cotangents [NV*d][NQ]
  static constexpr int VJP_PER = NV * NB + NV * NQ + DIM * NV * NQ;
  static constexpr size_t JVP_SMEM = (size_t(EPB) * JVP_PER + TABLES + NQ * NB) * 8;
  static constexpr size_t VJP_SMEM = (size_t(EPB) * VJP_PER + TABLES + NQ * NB) * 8 + 8 * 32;
  static constexpr size_t TRACE_SMEM = size_t(TABLES + NQ * NB) * 8;
  // gradient transpose (affine): lamTot and lamJmp [NV*2][NB] | phif | dmod | emod | lmod
  static constexpr int GOPS = NFP * NB + DIM * NB * NB + NF * NB * NFQ + NF * NFQ * NFQ;
  static constexpr size_t GRAD_SMEM = (size_t(EPB) * 2 * DIM * NV * NB + GOPS) * 8;
  // gradient transpose (general form): lamRt, lamRv [NV*2][NB] | lamRf [NF][NV*2][NB] | point values' cotangent
  // [NV][NQ] | phi | dphiw | phif | phifw | mref
  static constexpr size_t GRAD_GENERAL_SMEM = (size_t(EPB) * ((2 + NF) * 2 * NV * NB + NV * NQ) + TABLES) * 8;
};

// Geometry of point q of element e: contravariant metric, 1/|J| at the point; the M^-1 of the element and its
// scale (affine: M_ref^-1 and 1/|J|, bilinear: the element's own inverse and 1).
template <int NB, int NQ, bool AFFINE, int DIM = 2>
__device__ __forceinline__ const double* densePointGeom(const double* geom, int64_t e, int q) {
  constexpr int GD = DIM * DIM + 1, GS = AFFINE ? GD : NQ * GD + NB * NB;
  return AFFINE ? geom + e * GS : geom + e * GS + q * GD;
}

template <int NB, int NQ, int NFQ, int NF, int DIM = 2>
__device__ __forceinline__ void loadDenseAdjTables(double* tab, const double* src) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, DIM>;
  for (int k = threadIdx.x; k < S::TABLES; k += blockDim.x) tab[k] = src[k];
  for (int k = threadIdx.x; k < NQ * NB; k += blockDim.x) tab[S::TABLES + k] = src[S::PHIW + k];
}

// Tangent element kernel of a dense block: dR at the stage input u in direction du (face tangents in dflux), the
// rate tangent and / or the RK combination dout = c0 dbase + c1 du + c2dt s M^-1 dR with the traces of dout.
template <int NB, int NQ, int NFQ, int NF, bool AFFINE, bool VISC, int DIM = 2>
__global__ void __launch_bounds__(256) jvpDenseStageKernel(AdjArgs a, Phys ph) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, DIM>;
  constexpr int NV = DIM + 2, NFP = S::NFP, EPB = S::EPB, GD = DIM * DIM + 1, GS = AFFINE ? GD : NQ * GD + NB * NB;
  using D1 = Dual<1>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE]
  double* sD = sU + EPB * S::USTRIDE;                // [EPB][USTRIDE] tangent state (then the new tangent)
  double* sF = sD + EPB * S::USTRIDE;                // [EPB][FSTRIDE] tangent flux slots
  double* sQ = sF + EPB * S::FSTRIDE;                // [EPB][DIM][NV][NQ] tangent contravariant fluxes
  double* sS = sQ + EPB * DIM * NV * NQ;             // [EPB][NQ] tangent of the source S |J|
  double* sR = sS + EPB * NQ;                        // [EPB][NV][NB] tangent residual
  double* tab = sR + EPB * NV * NB;
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phif = dphiw + NQ * DIM * NB;
  const double* phifw = phif + NFP * NB;
  const double* mref = phifw + NFP * NB;
  const double* phiw = tab + S::TABLES;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF, DIM>(tab, a.tables);
  for (int k = tid; k < ecount * S::USTRIDE; k += blockDim.x) {
    sU[k] = a.u[e0 * S::USTRIDE + k];
    sD[k] = a.du[e0 * S::USTRIDE + k];
  }
  for (int k = tid; k < ecount * S::FSTRIDE; k += blockDim.x) sF[k] = a.dflux[(a.faceBase + e0 * NF) * NV * NFQ + k];
  __syncthreads();
  for (int idx = tid; idx < ecount * NQ; idx += blockDim.x) {
    const int le = idx / NQ, q = idx - le * NQ;
    const int64_t e = e0 + le;
    D1 U[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0, d = 0.0;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        s = fma(phi[q * NB + b], sU[le * S::USTRIDE + v * NB + b], s);
        d = fma(phi[q * NB + b], sD[le * S::USTRIDE + v * NB + b], d);
      }
      U[v].v = s; U[v].d[0] = d;
    }
    const double* g = densePointGeom<NB, NQ, AFFINE, DIM>(a.geom, e, q);
    double ja[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[r][c] = g[r * DIM + c];
    D1 gg[VISC ? NV * DIM : 1], Q[DIM][NV], Qv[DIM][NV];
    if constexpr (VISC) {  // the gradient at the point from the modal gradient coefficients and their tangent
#pragma unroll
      for (int c = 0; c < NV * DIM; ++c) {
        double x = 0.0, dx = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          x = fma(phi[q * NB + b], a.grad[(e * NV * DIM + c) * NB + b], x);
          dx = fma(phi[q * NB + b], a.dgrad[(e * NV * DIM + c) * NB + b], dx);
        }
        gg[c].v = x; gg[c].d[0] = dx;
      }
    }
    nodeFlux<DIM, VISC>(U, gg, ja, ph, Q, Qv);
    const double mscale = VISC && ph.mu > 0.0 ? a.dmu / ph.mu : 0.0;
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) sQ[((le * DIM + b) * NV + v) * NQ + q] = fma(mscale, Qv[b][v].v, Q[b][v].d[0]);
    if (ph.source) {
      State<DIM, D1> st;
      makeState<DIM>(st, U, ph);
      const D1 src = st.r * ph.beta * (temperatureOf(st, ph) - ph.tref);
      sS[le * NQ + q] = src.d[0] / g[DIM * DIM];
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
      for (int q = 0; q < NQ; ++q) {
#pragma unroll
        for (int b = 0; b < DIM; ++b) s = fma(sQ[((le * DIM + b) * NV + v) * NQ + q], dphiw[(q * DIM + b) * NB + i], s);
      }
      for (int fj = 0; fj < NFP; ++fj) {
        const int f = fj / NFQ, j = fj - f * NFQ;
        s = fma(-sF[le * S::FSTRIDE + (f * NV + v) * NFQ + j], phifw[fj * NB + i], s);
      }
      if (ph.source && v == DIM)
        for (int q = 0; q < NQ; ++q) s = fma(sS[le * NQ + q], phiw[q * NB + i], s);
      sR[(le * NV + v) * NB + i] = s;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GS;
    const double* minv = AFFINE ? mref : g + NQ * GD;
    const double sc = AFFINE ? g[DIM * DIM] : 1.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
      for (int k = 0; k < NB; ++k) s = fma(minv[i * NB + k], sR[(le * NV + v) * NB + k], s);
      const double ddu = sc * s;
      const int64_t gi = e * S::USTRIDE + v * NB + i;
      if (a.drate) a.drate[gi] = ddu;
      const double dn = fma(a.c2dt, ddu, fma(a.c1, sD[le * S::USTRIDE + v * NB + i], a.c0 * (a.dbase ? a.dbase[gi] : 0.0)));
      sQ[(le * NV + v) * NB + i] = dn;  // sQ reused: the new tangent per basis function
    }
  }
  __syncthreads();
  if (!a.dout) return;
  for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
    const int le = idx / (NV * NB), r = idx - le * NV * NB;
    a.dout[(e0 + le) * S::USTRIDE + r] = sQ[le * NV * NB + r];
  }
  if (!a.dtrace) return;
  for (int idx = tid; idx < ecount * NFP; idx += blockDim.x) {
    const int le = idx / NFP, fj = idx - le * NFP;
    const int f = fj / NFQ, j = fj - f * NFQ;
    double* out = a.dtrace + (a.faceBase + (e0 + le) * NF + f) * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
#pragma unroll
      for (int b = 0; b < NB; ++b) s = fma(phif[fj * NB + b], sQ[(le * NV + v) * NB + b], s);
      out[v * NFQ] = s;
    }
  }
}

// Adjoint of the volume and lift terms of a dense block: lamU (state layout) and lamH (the flux slots of the
// block's faces) from lam, the cotangent of du/dt.
template <int NB, int NQ, int NFQ, int NF, bool AFFINE, bool GEN, bool VISC, int DIM = 2>
__global__ void __launch_bounds__(256) vjpDenseVolumeKernel(AdjArgs a, Phys ph) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, DIM>;
  constexpr int NV = DIM + 2, NFP = S::NFP, EPB = S::EPB, GD = DIM * DIM + 1, GS = AFFINE ? GD : NQ * GD + NB * NB,
                NR = NV * DIM;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sL = reinterpret_cast<double*>(smem_raw);  // [EPB][NV][NB] lamR = s M^-T lam
  double* sP = sL + EPB * NV * NB;                   // [EPB][NV][NQ] point cotangents of U_q
  double* sPG = sP + EPB * NV * NQ;                  // [EPB][NR][NQ] point cotangents of G_q (Navier-Stokes)
  double* tab = sPG + EPB * NR * NQ;
  double* sRed = tab + S::TABLES + NQ * NB;          // one double per warp
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phifw = dphiw + NQ * DIM * NB + NFP * NB;
  const double* mref = phifw + NFP * NB;
  const double* phiw = tab + S::TABLES;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF, DIM>(tab, a.tables);
  __syncthreads();
  double mupart = 0.0;
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, k = idx - le * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GS;
    const double* minv = AFFINE ? mref : g + NQ * GD;
    const double sc = AFFINE ? g[DIM * DIM] : 1.0;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
      for (int i = 0; i < NB; ++i) s = fma(minv[i * NB + k], a.lam[e * S::USTRIDE + v * NB + i], s);
      sL[(le * NV + v) * NB + k] = sc * s;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NQ; idx += blockDim.x) {
    const int le = idx / NQ, q = idx - le * NQ;
    const int64_t e = e0 + le;
    double lq[DIM][NV];
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < NB; ++i) s = fma(dphiw[(q * DIM + b) * NB + i], sL[(le * NV + v) * NB + i], s);
        lq[b][v] = s;
      }
    double U[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
#pragma unroll
      for (int b = 0; b < NB; ++b) s = fma(phi[q * NB + b], a.u[e * S::USTRIDE + v * NB + b], s);
      U[v] = s;
    }
    const double* g = densePointGeom<NB, NQ, AFFINE, DIM>(a.geom, e, q);
    double ja[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[r][c] = g[r * DIM + c];
    double lu[NV], gg[VISC ? NR : 1], lg[VISC ? NR : 1];
    if constexpr (VISC) {
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        double x = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) x = fma(phi[q * NB + b], a.grad[(e * NR + c) * NB + b], x);
        gg[c] = x;
        lg[c] = 0.0;
      }
    }
    if constexpr (GEN) {
      // the source enters R as w_q |J|_q S(U_q) phi: its cotangent is |J|_q (phiw^T lamR)_q on the last momentum
      double lamS = 0.0;
      if (ph.source) {
#pragma unroll
        for (int i = 0; i < NB; ++i) lamS = fma(phiw[q * NB + i], sL[(le * NV + DIM) * NB + i], lamS);
        lamS /= g[DIM * DIM];
      }
      mupart += volumeReverseGeneric<DIM, VISC>(U, gg, ja, lq, lamS, ph, lu, lg);
    } else {
      eulerVolumeReverse<DIM>(U, ja, lq, ph, lu);
      if constexpr (VISC) {
        // lamF[c][v] = cotangent of Fv_c(v): Q_b contains -sum_c ja[b][c] Fv_c
        double lamF[DIM][NV];
#pragma unroll
        for (int c = 0; c < DIM; ++c)
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            double s = ja[DIM - 1][c] * lq[DIM - 1][v];
#pragma unroll
            for (int b = DIM - 2; b >= 0; --b) s = fma(ja[b][c], lq[b][v], s);
            lamF[c][v] = -s;
          }
        mupart += viscousReverse<DIM>(U, gg, lamF, ph, lu, lg);
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) sP[(le * NV + v) * NQ + q] = lu[v];
    if constexpr (VISC) {
#pragma unroll
      for (int c = 0; c < NR; ++c) sPG[(le * NR + c) * NQ + q] = lg[c];
    }
  }
  if constexpr (VISC) blockSum(mupart, a.muPart + blockIdx.x, sRed);
  __syncthreads();
  if constexpr (VISC) {  // lamw = Phi^T lamG_q
    for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
      const int le = idx / NB, i = idx - le * NB;
      const int64_t e = e0 + le;
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        double x = 0.0;
        for (int q = 0; q < NQ; ++q) x = fma(phi[q * NB + i], sPG[(le * NR + c) * NQ + q], x);
        a.lamG[(e * NR + c) * NB + i] = x;
      }
    }
  }
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
    const int64_t e = e0 + le;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
      for (int q = 0; q < NQ; ++q) s = fma(phi[q * NB + i], sP[(le * NV + v) * NQ + q], s);
      a.lamU[e * S::USTRIDE + v * NB + i] = s;
    }
  }
  // transposed lift: lamH(fj) = -Phifw_fj lamR
  for (int idx = tid; idx < ecount * NFP; idx += blockDim.x) {
    const int le = idx / NFP, fj = idx - le * NFP;
    const int f = fj / NFQ, j = fj - f * NFQ;
    double* out = a.lamH + (a.faceBase + (e0 + le) * NF + f) * NV * NFQ + j;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
#pragma unroll
      for (int i = 0; i < NB; ++i) s = fma(-phifw[fj * NB + i], sL[(le * NV + v) * NB + i], s);
      out[v * NFQ] = s;
    }
  }
}

// Transposed gradient pass of an affine dense block (denseGradientAffineTile).  Forward, per element:
//   tot_k = -sum_b ja[b][k] (D_b u) + sum_f nF_f[k] E_f O_f,   jmp_k = sum_f nF_f[k] E_f (O_f - S_f)/2
//   grad_k = jinv tot_k;  BR1: w_k = grad_k;  BR2: w_k = jinv (tot_k - jmp_k)
//   gradient trace at (f, j): (Phi_f w_k)_j (+ BR2: jinv nF_f[k] (L_f (O_f - S_f)/2)_j)
// with S the own traces and O the neighbour traces.  Transposed, with lamVol = Phi_f^T lamTg:
//   lamTot = jinv (lamG + lamVol),  lamJmp = -jinv lamVol (BR2),
//   lamU -= sum_b D_b^T (sum_k ja[b][k] lamTot_k),
//   lamO_f = E_f^T (nF_f . lamTot);  BR2: lamD_f = E_f^T (nF_f . lamJmp) + jinv L_f^T (nF_f . lamTg_f),
//   lamUp = lamO + lamD/2 (the neighbour traces), lamTr += -lamD/2 (the own traces).
template <int NB, int NQ, int NFQ, int NF, bool BR2, int DIM = 2>
__global__ void __launch_bounds__(256) vjpDenseGradientKernel(AdjArgs a) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, DIM>;
  constexpr int NV = DIM + 2, NFP = S::NFP, EPB = S::EPB, NR = NV * DIM, GD = DIM * DIM + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sT = reinterpret_cast<double*>(smem_raw);  // [EPB][NR][NB] lamTot
  double* sJ = sT + EPB * NR * NB;                   // [EPB][NR][NB] lamJmp (BR2)
  double* tab = sJ + EPB * NR * NB;
  const double* phif = tab;                          // [NFP][NB]
  const double* dmod = phif + NFP * NB;              // [DIM][NB][NB]
  const double* emod = dmod + DIM * NB * NB;         // [NF][NB][NFQ]
  const double* lmod = emod + NF * NB * NFQ;         // [NF][NFQ][NFQ]
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  {
    constexpr int OFF_PHIF = NQ * NB * (1 + DIM), OFF_DMOD = NQ * NB * (1 + DIM) + NFP * NB * 2 + NB * NB;
    constexpr int NOPS = DIM * NB * NB + NF * NB * NFQ + NF * NFQ * NFQ;
    for (int k = tid; k < NFP * NB; k += blockDim.x) tab[k] = a.tables[OFF_PHIF + k];
    for (int k = tid; k < NOPS; k += blockDim.x) tab[NFP * NB + k] = a.tables[OFF_DMOD + k];
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NR * NB; idx += blockDim.x) {
    const int le = idx / (NR * NB), r = idx - le * NR * NB;
    const int c = r / NB, i = r - c * NB;
    const int64_t e = e0 + le;
    const double jinv = a.geom[e * GD + DIM * DIM];
    double vol = 0.0;
    for (int fj = 0; fj < NFP; ++fj) {
      const int f = fj / NFQ, j = fj - f * NFQ;
      vol = fma(phif[fj * NB + i], a.lamTg[(a.faceBase + e * NF + f) * NR * NFQ + c * NFQ + j], vol);
    }
    sT[(le * NR + c) * NB + i] = jinv * (a.lamG[(e * NR + c) * NB + i] + vol);
    if constexpr (BR2) sJ[(le * NR + c) * NB + i] = -jinv * vol;
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
    const int le = idx / (NV * NB), r = idx - le * NV * NB;
    const int v = r / NB, m = r - v * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GD;
    double acc = 0.0;
    for (int i = 0; i < NB; ++i) {
      const double* t = sT + (le * NR + v * DIM) * NB + i;  // lamTot_k at stride NB
#pragma unroll
      for (int b = 0; b < DIM; ++b) {  // d_b = sum_k ja[b][k] lamTot_k
        double d = g[b * DIM + DIM - 1] * t[(DIM - 1) * NB];
#pragma unroll
        for (int kk = DIM - 2; kk >= 0; --kk) d = fma(g[b * DIM + kk], t[kk * NB], d);
        acc = fma(dmod[(b * NB + i) * NB + m], d, acc);
      }
    }
    a.lamU[e * S::USTRIDE + v * NB + m] -= acc;
  }
  for (int idx = tid; idx < ecount * NFP * NV; idx += blockDim.x) {
    const int le = idx / (NFP * NV), r = idx - le * NFP * NV;
    const int fj = r / NV, v = r - fj * NV;
    const int f = fj / NFQ, j = fj - f * NFQ;
    const int64_t e = e0 + le;
    const double jinv = a.geom[e * GD + DIM * DIM];
    const double* nf = a.fmetric + (a.fmetricPoint ? (e * NF + f) * NFQ + j : e * NF + f) * DIM;
    // n . x for components x_k at stride `st`
    const auto ndot = [&](const double* x, int st) {
      double r = nf[DIM - 1] * x[(DIM - 1) * st];
#pragma unroll
      for (int kk = DIM - 2; kk >= 0; --kk) r = fma(nf[kk], x[kk * st], r);
      return r;
    };
    double lo = 0.0, ld = 0.0;
    for (int i = 0; i < NB; ++i) {
      const double E = emod[(f * NB + i) * NFQ + j];
      lo = fma(E, ndot(sT + (le * NR + v * DIM) * NB + i, NB), lo);
      if constexpr (BR2) ld = fma(E, ndot(sJ + (le * NR + v * DIM) * NB + i, NB), ld);
    }
    const int64_t slot = (a.faceBase + e * NF + f);
    if constexpr (BR2) {
      const double* tg = a.lamTg + slot * NR * NFQ;
      double lift = 0.0;
#pragma unroll
      for (int jj = 0; jj < NFQ; ++jj)
        lift = fma(lmod[(f * NFQ + jj) * NFQ + j], ndot(tg + v * DIM * NFQ + jj, NFQ), lift);
      ld = fma(jinv, lift, ld);
      a.lamTr[slot * NV * NFQ + v * NFQ + j] += -0.5 * ld;
    }
    a.lamUp[slot * NV * NFQ + v * NFQ + j] = fma(0.5, ld, lo);
  }
}

// Transposed gradient pass of a bilinear dense block (denseGradientTile's general form: per-point metric g_q, the
// element's own M^-1).  Forward, per variable with the face points' weighted values phifw:
//   Rt_k = sum_fj phifw_fj O_fj nF_f[k] - sum_q U_q sum_b dphiw_qb g_q[b][k],   Rv_k: (O + S)/2 in place of O
//   grad = M^-1 Rt;  BR1 gradient traces Phi_f grad;  BR2: Phi_f (M^-1 Rv + M^-1 Rf_f) with
//   Rf_f,k = sum_{j in f} phifw_fj (O - S)_fj / 2 nF_f[k].
// Transposed: lamRt = M^-T (lamG + [BR1] Phi_f^T lamTg), BR2: lamRv = M^-T Phi_f^T lamTg over all faces and
// lamRf_f = M^-T Phi_f^T lamTg over face f's points; then the points' values, O (lamUp) and S (lamTr, BR2).
template <int NB, int NQ, int NFQ, int NF, bool BR2>
__global__ void __launch_bounds__(256) vjpDenseGradientGeneralKernel(AdjArgs a) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  constexpr int NV = 4, NFP = S::NFP, EPB = S::EPB, NR = NV * 2, GS = NQ * 5 + NB * NB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sRt = reinterpret_cast<double*>(smem_raw);  // [EPB][NR][NB] lamRt
  double* sRv = sRt + EPB * NR * NB;                  // [EPB][NR][NB] lamRv (BR2)
  double* sRf = sRv + EPB * NR * NB;                  // [EPB][NF][NR][NB] lamRf (BR2)
  double* sUq = sRf + EPB * NF * NR * NB;             // [EPB][NV][NQ] cotangent of the point values
  double* tab = sUq + EPB * NV * NQ;
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phif = dphiw + NQ * 2 * NB;
  const double* phifw = phif + NFP * NB;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  for (int k = tid; k < S::TABLES; k += blockDim.x) tab[k] = a.tables[k];
  __syncthreads();
  // lamRt, lamRv, lamRf = M^-T (...) per (element, component, basis function)
  for (int idx = tid; idx < ecount * NR * NB; idx += blockDim.x) {
    const int le = idx / (NR * NB), r = idx - le * NR * NB;
    const int c = r / NB, m = r - c * NB;
    const int64_t e = e0 + le;
    const double* minv = a.geom + e * GS + NQ * 5;
    const double* tg = a.lamTg + (a.faceBase + e * NF) * NR * NFQ;
    double t = 0.0, v = 0.0, fsum[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) fsum[f] = 0.0;
    for (int i = 0; i < NB; ++i) {
      double trf[NF];  // (Phi_f^T lamTg_f)(i) per face
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        double x = 0.0;
#pragma unroll
        for (int j = 0; j < NFQ; ++j) x = fma(phif[(f * NFQ + j) * NB + i], tg[(f * NR + c) * NFQ + j], x);
        trf[f] = x;
      }
      double all = 0.0;
#pragma unroll
      for (int f = 0; f < NF; ++f) all += trf[f];
      const double mi = minv[i * NB + m];
      t = fma(mi, a.lamG[(e * NR + c) * NB + i] + (BR2 ? 0.0 : all), t);
      if constexpr (BR2) {
        v = fma(mi, all, v);
#pragma unroll
        for (int f = 0; f < NF; ++f) fsum[f] = fma(mi, trf[f], fsum[f]);
      }
    }
    sRt[(le * NR + c) * NB + m] = t;
    if constexpr (BR2) {
      sRv[(le * NR + c) * NB + m] = v;
#pragma unroll
      for (int f = 0; f < NF; ++f) sRf[((le * NF + f) * NR + c) * NB + m] = fsum[f];
    }
  }
  __syncthreads();
  // the points' values: lamUq = -sum_k sum_b g_q[b][k] sum_i dphiw_qb(i) (lamRt + lamRv)_k(i)
  for (int idx = tid; idx < ecount * NV * NQ; idx += blockDim.x) {
    const int le = idx / (NV * NQ), r = idx - le * NV * NQ;
    const int v = r / NQ, q = r - v * NQ;
    const double* g = a.geom + (e0 + le) * GS + q * 5;
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        double x = 0.0;
#pragma unroll
        for (int i = 0; i < NB; ++i) {
          const double l = sRt[(le * NR + v * 2 + k) * NB + i] + (BR2 ? sRv[(le * NR + v * 2 + k) * NB + i] : 0.0);
          x = fma(dphiw[(q * 2 + b) * NB + i], l, x);
        }
        acc = fma(g[b * 2 + k], x, acc);
      }
    sUq[(le * NV + v) * NQ + q] = -acc;
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
    const int le = idx / (NV * NB), r = idx - le * NV * NB;
    const int v = r / NB, m = r - v * NB;
    double acc = 0.0;
    for (int q = 0; q < NQ; ++q) acc = fma(phi[q * NB + m], sUq[(le * NV + v) * NQ + q], acc);
    a.lamU[(e0 + le) * S::USTRIDE + v * NB + m] += acc;
  }
  // the traces: O from Rt (and Rv / 2, Rf / 2), S from Rv / 2 and -Rf / 2
  for (int idx = tid; idx < ecount * NFP * NV; idx += blockDim.x) {
    const int le = idx / (NFP * NV), r = idx - le * NFP * NV;
    const int fj = r / NV, v = r - fj * NV;
    const int f = fj / NFQ, j = fj - f * NFQ;
    const int64_t e = e0 + le;
    const double* nfp = a.fmetric + (a.fmetricPoint ? (e * NF + f) * NFQ + j : e * NF + f) * 2;
    const double n0 = nfp[0], n1 = nfp[1];
    double lt = 0.0, lv = 0.0, lf = 0.0;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
      const double w = phifw[fj * NB + i];
      lt = fma(w, fma(n0, sRt[(le * NR + v * 2) * NB + i], n1 * sRt[(le * NR + v * 2 + 1) * NB + i]), lt);
      if constexpr (BR2) {
        lv = fma(w, fma(n0, sRv[(le * NR + v * 2) * NB + i], n1 * sRv[(le * NR + v * 2 + 1) * NB + i]), lv);
        lf = fma(w, fma(n0, sRf[((le * NF + f) * NR + v * 2) * NB + i], n1 * sRf[((le * NF + f) * NR + v * 2 + 1) * NB + i]), lf);
      }
    }
    const int64_t slot = a.faceBase + e * NF + f;
    a.lamUp[slot * NV * NFQ + v * NFQ + j] = BR2 ? lt + 0.5 * (lv + lf) : lt;
    if constexpr (BR2) a.lamTr[slot * NV * NFQ + v * NFQ + j] += 0.5 * (lv - lf);
  }
}

// lamU += Phi_f^T lamTr over the block's face points, then the RK combination of the stage's cotangents (the
// tensor vjpTraceKernel's rule).
template <int NB, int NQ, int NFQ, int NF, int DIM = 2>
__global__ void __launch_bounds__(256) vjpDenseTraceKernel(AdjArgs a) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, DIM>;
  constexpr int NV = DIM + 2, NFP = S::NFP, EPB = S::EPB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  const double* phif = tab + NQ * NB * (1 + DIM);
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF, DIM>(tab, a.tables);
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
    const int64_t e = e0 + le;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int64_t gi = e * S::USTRIDE + v * NB + i;
      double lu = a.lamU[gi];
      for (int fj = 0; fj < NFP; ++fj) {
        const int f = fj / NFQ, j = fj - f * NFQ;
        lu = fma(phif[fj * NB + i], a.lamTr[(a.faceBase + e * NF + f) * NV * NFQ + v * NFQ + j], lu);
      }
      const double li = a.lamIn ? a.lamIn[gi] : 0.0;
      if (a.accumulateAll) {
        a.lamBase[gi] += fma(a.c2dt, lu, (a.c0 + a.c1) * li);
      } else {
        if (a.lamStage) a.lamStage[gi] = fma(a.c2dt, lu, a.c1 * li);
        if (a.lamBase) a.lamBase[gi] += a.c0 * li;
        if (!a.lamStage && !a.lamBase) a.lamU[gi] = lu;
      }
    }
  }
}

}  // namespace sdg
