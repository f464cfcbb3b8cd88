// Tangent-linear (JVP) and adjoint (VJP) element kernels of dense (modal) blocks -- triangles and first-order
// quadrangles, affine or bilinear -- for the Euler equations (compressible or incompressible, with the
// Boussinesq source).  The face kernels of sdg_kernels_adjoint.cuh serve these blocks unchanged: they work on
// the face slots, whose layout [slot][nv][nfq] is the same for every block kind.
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
#pragma once
#include "sdg_kernels_adjoint.cuh"
#include "sdg_kernels_dense.cuh"

namespace sdg {

template <int NB, int NQ, int NFQ, int NF>
struct DenseAdjShape {
  static constexpr int NV = 4, NFP = NF * NFQ;
  static constexpr int USTRIDE = (NV * NB + 1) & ~1;
  static constexpr int FSTRIDE = NF * NV * NFQ;
  static constexpr int EPB = 8, THREADS = 256;
  // phi | dphiw | phif | phifw | mref (the forward dense tables' leading part) | phiw (volume source weights)
  static constexpr int TABLES = NQ * NB * 3 + NFP * NB * 2 + NB * NB;
  static constexpr int PHIW = NQ * NB * 3 + NFP * NB * 2 + NB * NB + 2 * NB * NB + NF * NB * NFQ + NF * NFQ * NFQ;
  // tangent: u, du | tangent flux slots | tangent fluxes [2][NV][NQ] | tangent source [NQ] | tangent residual
  static constexpr int JVP_PER = 2 * USTRIDE + FSTRIDE + 2 * NV * NQ + NQ + NV * NB;
  // adjoint: lamR [NV][NB] | point cotangents [NV][NQ]
  static constexpr int VJP_PER = NV * NB + NV * NQ;
  static constexpr size_t JVP_SMEM = (size_t(EPB) * JVP_PER + TABLES + NQ * NB) * 8;
  static constexpr size_t VJP_SMEM = (size_t(EPB) * VJP_PER + TABLES + NQ * NB) * 8;
  static constexpr size_t TRACE_SMEM = size_t(TABLES + NQ * NB) * 8;
};

// Geometry of point q of element e: contravariant metric, 1/|J| at the point; the M^-1 of the element and its
// scale (affine: M_ref^-1 and 1/|J|, bilinear: the element's own inverse and 1).
template <int NB, int NQ, bool AFFINE>
__device__ __forceinline__ const double* densePointGeom(const double* geom, int64_t e, int q) {
  constexpr int GS = AFFINE ? 5 : NQ * 5 + NB * NB;
  return AFFINE ? geom + e * GS : geom + e * GS + q * 5;
}

template <int NB, int NQ, int NFQ, int NF>
__device__ __forceinline__ void loadDenseAdjTables(double* tab, const double* src) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  for (int k = threadIdx.x; k < S::TABLES; k += blockDim.x) tab[k] = src[k];
  for (int k = threadIdx.x; k < NQ * NB; k += blockDim.x) tab[S::TABLES + k] = src[S::PHIW + k];
}

// Tangent element kernel of a dense block: dR at the stage input u in direction du (face tangents in dflux), the
// rate tangent and / or the RK combination dout = c0 dbase + c1 du + c2dt s M^-1 dR with the traces of dout.
template <int NB, int NQ, int NFQ, int NF, bool AFFINE>
__global__ void __launch_bounds__(256) jvpDenseStageKernel(AdjArgs a, Phys ph) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  constexpr int NV = 4, NFP = S::NFP, EPB = S::EPB, GS = AFFINE ? 5 : NQ * 5 + NB * NB;
  using D1 = Dual<1>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE]
  double* sD = sU + EPB * S::USTRIDE;                // [EPB][USTRIDE] tangent state (then the new tangent)
  double* sF = sD + EPB * S::USTRIDE;                // [EPB][FSTRIDE] tangent flux slots
  double* sQ = sF + EPB * S::FSTRIDE;                // [EPB][2][NV][NQ] tangent contravariant fluxes
  double* sS = sQ + EPB * 2 * NV * NQ;               // [EPB][NQ] tangent of the source S |J|
  double* sR = sS + EPB * NQ;                        // [EPB][NV][NB] tangent residual
  double* tab = sR + EPB * NV * NB;
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phif = dphiw + NQ * 2 * NB;
  const double* phifw = phif + NFP * NB;
  const double* mref = phifw + NFP * NB;
  const double* phiw = tab + S::TABLES;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF>(tab, a.tables);
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
    const double* g = densePointGeom<NB, NQ, AFFINE>(a.geom, e, q);
    const double ja[2][2] = {{g[0], g[1]}, {g[2], g[3]}};
    D1 gg[1], Q[2][NV], Qv[2][NV];
    nodeFlux<2, false>(U, gg, ja, ph, Q, Qv);
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) sQ[((le * 2 + b) * NV + v) * NQ + q] = Q[b][v].d[0];
    if (ph.source) {
      State<2, D1> st;
      makeState<2>(st, U, ph);
      const D1 src = st.r * ph.beta * (temperatureOf(st, ph) - ph.tref);
      sS[le * NQ + q] = src.d[0] / g[4];
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double s = 0.0;
      for (int q = 0; q < NQ; ++q) {
        s = fma(sQ[((le * 2 + 0) * NV + v) * NQ + q], dphiw[(q * 2 + 0) * NB + i], s);
        s = fma(sQ[((le * 2 + 1) * NV + v) * NQ + q], dphiw[(q * 2 + 1) * NB + i], s);
      }
      for (int fj = 0; fj < NFP; ++fj) {
        const int f = fj / NFQ, j = fj - f * NFQ;
        s = fma(-sF[le * S::FSTRIDE + (f * NV + v) * NFQ + j], phifw[fj * NB + i], s);
      }
      if (ph.source && v == 2)
        for (int q = 0; q < NQ; ++q) s = fma(sS[le * NQ + q], phiw[q * NB + i], s);
      sR[(le * NV + v) * NB + i] = s;
    }
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, i = idx - le * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GS;
    const double* minv = AFFINE ? mref : g + NQ * 5;
    const double sc = AFFINE ? g[4] : 1.0;
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
template <int NB, int NQ, int NFQ, int NF, bool AFFINE, bool GEN>
__global__ void __launch_bounds__(256) vjpDenseVolumeKernel(AdjArgs a, Phys ph) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  constexpr int NV = 4, NFP = S::NFP, EPB = S::EPB, GS = AFFINE ? 5 : NQ * 5 + NB * NB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sL = reinterpret_cast<double*>(smem_raw);  // [EPB][NV][NB] lamR = s M^-T lam
  double* sP = sL + EPB * NV * NB;                   // [EPB][NV][NQ] point cotangents of U_q
  double* tab = sP + EPB * NV * NQ;
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phifw = dphiw + NQ * 2 * NB + NFP * NB;
  const double* mref = phifw + NFP * NB;
  const double* phiw = tab + S::TABLES;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF>(tab, a.tables);
  __syncthreads();
  for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
    const int le = idx / NB, k = idx - le * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GS;
    const double* minv = AFFINE ? mref : g + NQ * 5;
    const double sc = AFFINE ? g[4] : 1.0;
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
    double lq[2][NV];
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < NB; ++i) s = fma(dphiw[(q * 2 + b) * NB + i], sL[(le * NV + v) * NB + i], s);
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
    const double* g = densePointGeom<NB, NQ, AFFINE>(a.geom, e, q);
    const double ja[2][2] = {{g[0], g[1]}, {g[2], g[3]}};
    double lu[NV];
    if constexpr (GEN) {
      // the source enters R as w_q |J|_q S(U_q) phi: its cotangent is |J|_q (phiw^T lamR)_q on the last momentum
      double lamS = 0.0;
      if (ph.source) {
#pragma unroll
        for (int i = 0; i < NB; ++i) lamS = fma(phiw[q * NB + i], sL[(le * NV + 2) * NB + i], lamS);
        lamS /= g[4];
      }
      double gg[1], lg[1];
      volumeReverseGeneric<2, false>(U, gg, ja, lq, lamS, ph, lu, lg);
    } else {
      eulerVolumeReverse<2>(U, ja, lq, ph, lu);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) sP[(le * NV + v) * NQ + q] = lu[v];
  }
  __syncthreads();
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

// lamU += Phi_f^T lamTr over the block's face points, then the RK combination of the stage's cotangents (the
// tensor vjpTraceKernel's rule).
template <int NB, int NQ, int NFQ, int NF>
__global__ void __launch_bounds__(256) vjpDenseTraceKernel(AdjArgs a) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  constexpr int NV = 4, NFP = S::NFP, EPB = S::EPB;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* tab = reinterpret_cast<double*>(smem_raw);
  const double* phif = tab + NQ * NB * 3;
  const int tid = threadIdx.x;
  const int64_t e0 = int64_t(blockIdx.x) * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  loadDenseAdjTables<NB, NQ, NFQ, NF>(tab, a.tables);
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
