// Dense (modal) element blocks and point-layout conversion kernels of the GB300 DG path.
//
// Triangles, and quadrangles of order 1 (whose volume rule is the non-tensor 7-point formula of
// src/Solver/SimulationControl.cpp:270), keep the reference's modal formulation
// (src/Solver/SpatialDiscrete.cpp:194-266,1016-1032; src/Solver/TimeIntegration.cpp:181-198): the state
// is the modal coefficient vector, the residual is R = sum_q Q_q grad(phi)_q - sum_j F_j phi_j with the
// operator tables staged in shared memory, and M^-1 is M_ref^-1/|J| on affine elements (an exact
// identity of the quadrature mass matrix) or a per-element inverse on bilinear quadrangles.
#pragma once
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "sdg_kernels.cuh"
#include "sdg_mesh.hpp"
#include "sdg_operators.hpp"

namespace sdg {

// Table layout (doubles, d = 2, or 3 on tetrahedra): phi[NQ][NB] | dphiw[NQ][d][NB] (w_q dphi/dxi_b) | phif[NFP][NB] |
//                         phifw[NFP][NB] (wf_j phif) | mref[NB][NB] (inverse reference mass matrix) |
//   modal gradient operators of affine elements (M = |J| M_ref folds M^-1 into them):
//                         dmod[d][NB][NB]  D_b = M_ref^-1 S_b, S_b(k,m) = sum_q w_q dphi_k/dxi_b phi_m
//                         emod[NF][NB][NFQ] E_f = M_ref^-1 Phi_f^T W_f (lift of face f's point values)
//                         lmod[NF][NFQ][NFQ] L_f = Phi_f E_f (trace at face f of the lift from face f)
//   source weights:        phiw[NQ][NB] w_q phi (volume source terms)
__host__ __device__ constexpr inline size_t denseTableSize(int nb, int nq, int nfp, int dim = 2) {
  return size_t(nq) * nb * (1 + dim) + size_t(nfp) * nb * 2 + size_t(nb) * nb;
}
__host__ __device__ constexpr inline size_t denseGradOperatorSize(int nb, int nf, int nfq, int dim = 2) {
  return size_t(dim) * nb * nb + size_t(nf) * nb * nfq + size_t(nf) * nfq * nfq;
}
__host__ __device__ constexpr inline size_t denseSourceTableOffset(int nb, int nq, int nfp, int nf, int nfq, int dim = 2) {
  return denseTableSize(nb, nq, nfp, dim) + denseGradOperatorSize(nb, nf, nfq, dim);
}
// Stage tables of affine blocks, M_ref^-1 folded in: phi[NQ][NB] | dphiwM[NQ][d][NB] | phif[NFP][NB] |
// phifwM[NFP][NB] | phiMr[NQ][NB], then phiwM[NQ][NB] (source weights).  dphiwM and phifwM are the weak
// derivative and face-lift tables with M_ref^-1 applied (the residual pass yields M_ref^-1 R directly: the
// affine M^-1 = M_ref^-1/|J| costs no N_b x N_b product per element); phiMr = Phi M_ref recovers R Phi^T from
// M_ref^-1 R for the relative error.
__host__ __device__ constexpr inline size_t denseFoldedOffset(int nb, int nq, int nfp, int nf, int nfq, int dim = 2) {
  return denseSourceTableOffset(nb, nq, nfp, nf, nfq, dim) + size_t(nq) * nb;
}
__host__ __device__ constexpr inline size_t denseFoldedSize(int nb, int nq, int nfp, int dim = 2) {
  return size_t(nq) * nb * (2 + dim) + size_t(nfp) * nb * 2;
}

template <class R>
inline void invertDense(int n, std::vector<R> a, std::vector<R>& inv) {
  inv.assign(size_t(n) * n, R(0));
  for (int i = 0; i < n; ++i) inv[size_t(i) * n + i] = R(1);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r) if (std::fabs(a[size_t(r) * n + c]) > std::fabs(a[size_t(piv) * n + c])) piv = r;
    for (int k = 0; k < n; ++k) { std::swap(a[size_t(c) * n + k], a[size_t(piv) * n + k]); std::swap(inv[size_t(c) * n + k], inv[size_t(piv) * n + k]); }
    const R d = R(1) / a[size_t(c) * n + c];
    for (int k = 0; k < n; ++k) { a[size_t(c) * n + k] *= d; inv[size_t(c) * n + k] *= d; }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const R f = a[size_t(r) * n + c];
      if (f == R(0)) continue;
      for (int k = 0; k < n; ++k) { a[size_t(r) * n + k] -= f * a[size_t(c) * n + k]; inv[size_t(r) * n + k] -= f * inv[size_t(c) * n + k]; }
    }
  }
}

void facePointInParent(int type, int f, const double* fx, double* X);

inline void buildDenseTables(int type, int p, std::vector<double>& tables, std::vector<double>& phiOut,
                             std::vector<double>& lsqOut) {
  const int nb = modalCount(type, p);
  const PointRule vr = volumeRule(type, p), fr = faceRule(type, p);
  const int nq = vr.n, nf = typeFaces(type), nfq = fr.n, nfp = nf * nfq, dim = typeDim(type);
  tables.assign(denseFoldedOffset(nb, nq, nfp, nf, nfq, dim) + denseFoldedSize(nb, nq, nfp, dim) + size_t(nq) * nb,
                0.0);
  double* phi = tables.data();
  double* dphiw = phi + size_t(nq) * nb;
  double* phif = dphiw + size_t(nq) * dim * nb;
  double* phifw = phif + size_t(nfp) * nb;
  double* mref = phifw + size_t(nfp) * nb;
  std::vector<double> v(nb), g(size_t(nb) * 3);
  for (int q = 0; q < nq; ++q) {
    modalBasis(type, p, &vr.x[q * 3], v.data(), g.data());
    for (int b = 0; b < nb; ++b) {
      phi[size_t(q) * nb + b] = v[b];
      for (int k = 0; k < dim; ++k) dphiw[(size_t(q) * dim + k) * nb + b] = vr.w[q] * g[b * 3 + k];
    }
  }
  for (int f = 0; f < nf; ++f)
    for (int j = 0; j < nfq; ++j) {
      double X[3]; facePointInParent(type, f, &fr.x[j * 3], X);
      modalBasis(type, p, X, v.data(), g.data());
      for (int b = 0; b < nb; ++b) {
        phif[size_t(f * nfq + j) * nb + b] = v[b];
        phifw[size_t(f * nfq + j) * nb + b] = fr.w[j] * v[b];
      }
    }
  // reference mass matrix and Phi^T Phi, and their inverses, in long double (rounded once to double)
  std::vector<long double> m(size_t(nb) * nb, 0.0L), ptp(size_t(nb) * nb, 0.0L), invl;
  for (int a = 0; a < nb; ++a)
    for (int b = 0; b < nb; ++b) {
      long double s = 0, t = 0;
      for (int q = 0; q < nq; ++q) {
        const long double pa = phi[size_t(q) * nb + a], pb = phi[size_t(q) * nb + b];
        s += (long double)vr.w[q] * pa * pb;
        t += pa * pb;
      }
      m[size_t(a) * nb + b] = s; ptp[size_t(a) * nb + b] = t;
    }
  invertDense(nb, m, invl);
  std::vector<double> inv(invl.begin(), invl.end());
  std::copy(inv.begin(), inv.end(), mref);
  {
    double* dmod = mref + size_t(nb) * nb;
    double* emod = dmod + size_t(dim) * nb * nb;
    double* lmod = emod + size_t(nf) * nb * nfq;
    for (int b = 0; b < dim; ++b) {
      std::vector<long double> sb(size_t(nb) * nb, 0.0L);
      for (int k = 0; k < nb; ++k)
        for (int mm = 0; mm < nb; ++mm) {
          long double acc = 0.0L;
          for (int q = 0; q < nq; ++q)
            acc += (long double)dphiw[(size_t(q) * dim + b) * nb + k] * (long double)phi[size_t(q) * nb + mm];
          sb[size_t(k) * nb + mm] = acc;
        }
      for (int i = 0; i < nb; ++i)
        for (int mm = 0; mm < nb; ++mm) {
          long double acc = 0.0L;
          for (int k = 0; k < nb; ++k) acc += (long double)inv[size_t(i) * nb + k] * sb[size_t(k) * nb + mm];
          dmod[(size_t(b) * nb + i) * nb + mm] = double(acc);
        }
    }
    std::vector<long double> ef(size_t(nf) * nb * nfq, 0.0L);
    for (int f = 0; f < nf; ++f)
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nfq; ++j) {
          long double acc = 0.0L;
          for (int k = 0; k < nb; ++k)
            acc += (long double)inv[size_t(i) * nb + k] * (long double)phifw[size_t(f * nfq + j) * nb + k];
          ef[(size_t(f) * nb + i) * nfq + j] = acc;
          emod[(size_t(f) * nb + i) * nfq + j] = double(acc);
        }
    for (int f = 0; f < nf; ++f)
      for (int j = 0; j < nfq; ++j)
        for (int jj = 0; jj < nfq; ++jj) {
          long double acc = 0.0L;
          for (int i = 0; i < nb; ++i)
            acc += (long double)phif[size_t(f * nfq + j) * nb + i] * ef[(size_t(f) * nb + i) * nfq + jj];
          lmod[(size_t(f) * nfq + j) * nfq + jj] = double(acc);
        }
  }
  {
    double* phiw = tables.data() + denseSourceTableOffset(nb, nq, nfp, nf, nfq, dim);
    for (int q = 0; q < nq; ++q)
      for (int b = 0; b < nb; ++b) phiw[size_t(q) * nb + b] = vr.w[q] * phi[size_t(q) * nb + b];
  }
  {
    // affine stage tables with M_ref^-1 folded in (long double sums of the long double inverse, rounded once)
    const double* phiw = tables.data() + denseSourceTableOffset(nb, nq, nfp, nf, nfq, dim);
    double* fo = tables.data() + denseFoldedOffset(nb, nq, nfp, nf, nfq, dim);
    double* fphi = fo;
    double* fdphiw = fphi + size_t(nq) * nb;
    double* fphif = fdphiw + size_t(nq) * dim * nb;
    double* fphifw = fphif + size_t(nfp) * nb;
    double* fphiM = fphifw + size_t(nfp) * nb;
    double* fphiw = fphiM + size_t(nq) * nb;
    // row r of `src` ([rows][nb]) times M_ref^-1 (symmetric): out[r][i] = sum_k inv[i][k] src[r][k]
    const auto fold = [&](const double* src, int rows, double* out) {
      for (int r = 0; r < rows; ++r)
        for (int i = 0; i < nb; ++i) {
          long double acc = 0.0L;
          for (int k = 0; k < nb; ++k) acc += invl[size_t(i) * nb + k] * (long double)src[size_t(r) * nb + k];
          out[size_t(r) * nb + i] = double(acc);
        }
    };
    std::copy(phi, phi + size_t(nq) * nb, fphi);
    fold(dphiw, nq * dim, fdphiw);
    std::copy(phif, phif + size_t(nfp) * nb, fphif);
    fold(phifw, nfp, fphifw);
    fold(phiw, nq, fphiw);
    for (int q = 0; q < nq; ++q)
      for (int k = 0; k < nb; ++k) {
        long double acc = 0.0L;
        for (int i = 0; i < nb; ++i) acc += (long double)phi[size_t(q) * nb + i] * m[size_t(i) * nb + k];
        fphiM[size_t(q) * nb + k] = double(acc);
      }
  }
  phiOut.assign(phi, phi + size_t(nq) * nb);
  // unweighted least-squares projection (InitialCondition.cpp:91-104): lsq = (Phi^T Phi)^-1 Phi^T  [nb][nq],
  // followed by its row sums [nb] (lsq applied to the constant 1: 1/phi_0 for the constant mode, 0 otherwise),
  // which let the projection act on u - u_ref and add u_ref back exactly
  invertDense(nb, ptp, invl);
  lsqOut.assign(size_t(nb) * nq + nb, 0.0);
  for (int b = 0; b < nb; ++b) {
    long double row = 0.0L;
    for (int q = 0; q < nq; ++q) {
      long double s = 0;
      for (int k = 0; k < nb; ++k) s += invl[size_t(b) * nb + k] * (long double)phi[size_t(q) * nb + k];
      lsqOut[size_t(b) * nq + q] = double(s);
      row += s;
    }
    lsqOut[size_t(nb) * nq + b] = double(row);
  }
}

template <int NB, int NQ, int NFQ, int NF, int DIM = 2>
struct DenseShape {
  static constexpr int NV = DIM + 2;
  static constexpr int NFP = NF * NFQ;
  static constexpr int USTRIDE = (NV * NB + 1) & ~1;
  static constexpr int FSTRIDE = NF * NV * NFQ;
  static_assert(DIM * NQ >= NB && NV * NB >= NQ, "shared-memory reuse of the point and coefficient buffers");
  static constexpr int PER_ELEM = USTRIDE + FSTRIDE + DIM * NV * NQ + NV * NB + NV * NB;
  // staged tables: bilinear blocks the original layout (M^-1 per element), affine blocks the folded one
  static constexpr size_t TABLES = size_t(NQ) * NB * (1 + DIM) + size_t(NFP) * NB * 2 + size_t(NB) * NB;
  static constexpr size_t TABLES_AFF = size_t(NQ) * NB * (2 + DIM) + size_t(NFP) * NB * 2;
  // tables above 160 KB (tetrahedra P5: 377 KB) are read in place from global memory (L2-resident, shared by
  // every CTA) instead of being staged per CTA
  static constexpr bool GLOBAL_TABLES = TABLES_AFF * 8 > 160 * 1024;
  __host__ __device__ static constexpr size_t tables(bool affine) {
    return affine ? (GLOBAL_TABLES ? 0 : TABLES_AFF) : TABLES;
  }
  static constexpr size_t TABLES_MAX_ = GLOBAL_TABLES ? 0 : TABLES_AFF + size_t(NB) * NB;
  // 16 elements per CTA, fewer where the tile and its tables would exceed the 227 KB opt-in shared memory
  static constexpr long long EPB_FIT =
      (227LL * 1024 - 16 - 8LL * NV * 8 - (long long)TABLES_MAX_ * 8) / ((long long)PER_ELEM * 8);
  static constexpr int EPB = EPB_FIT < 16 ? (EPB_FIT > 0 ? int(EPB_FIT) : 1) : 16;
  static constexpr int THREADS = 256;
  static constexpr size_t smemFor(int epb, int threads, bool affine) {
    return (size_t(epb) * PER_ELEM + tables(affine)) * 8 + 16 + 8 * NV * size_t(threads / 32);
  }
};

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
__device__ __forceinline__ uint64_t* denseStageBarrier(int epb) {
  using S = DenseShape<NB, NQ, NFQ, NF, DIM>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  return reinterpret_cast<uint64_t*>(reinterpret_cast<double*>(smem_raw) + epb * S::PER_ELEM + S::tables(AFFINE));
}

// Dense stage tile (triangles and P1 quadrangles: DIM 2; tetrahedra: DIM 3), a.epb elements per CTA, any
// whole number of warps.  geometry: affine [e][d*d+1] = (|J| dxi_b/dx_a row-major, 1/|J|); bilinear:
// [e][NQ][d*d+1] followed by the element's M^-1 [NB][NB].
template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int VISC, int DIM = 2>
__device__ __forceinline__ bool denseStageTile(const StageArgs& a, const Phys& ph, int64_t tile, uint32_t parity,
                                               bool loadTables) {
  using S = DenseShape<NB, NQ, NFQ, NF, DIM>;
  constexpr int NV = DIM + 2, NFP = S::NFP, GD = DIM * DIM + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int EPB = a.epb;
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE]
  double* sF = sU + EPB * S::USTRIDE;                // [EPB][FSTRIDE]
  double* sQ = sF + EPB * S::FSTRIDE;                // [EPB][DIM][NV][NQ]
  double* sR = sQ + EPB * DIM * NV * NQ;             // [EPB][NV][NB]
  double* sN = sR + EPB * NV * NB;                   // [EPB][NV][NB] new state
  double* tab = sN + EPB * NV * NB;
  // affine: the folded tables (dphiw and phifw carry M_ref^-1; the last block is phiMr = Phi M_ref), staged in
  // shared memory or, when too large, read in place (GT)
  constexpr size_t TAB = S::tables(AFFINE);
  constexpr bool GT = AFFINE && S::GLOBAL_TABLES;
  const double* tsrc = AFFINE ? a.tables + denseFoldedOffset(NB, NQ, NFP, NF, NFQ, DIM) : a.tables;
  const double* phi = GT ? tsrc : tab;
  const double* dphiw = phi + NQ * NB;
  const double* phif = dphiw + NQ * DIM * NB;
  const double* phifw = phif + NFP * NB;
  const double* mref = phifw + NFP * NB;  // affine: phiMr [NQ][NB]
  uint64_t* bar = reinterpret_cast<uint64_t*>(tab + TAB);
  double* sRed = reinterpret_cast<double*>(bar + 1);
  const int GS = AFFINE ? GD : NQ * GD + NB * NB;

  const int tid = threadIdx.x;
  const int64_t e0 = tile * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  __syncthreads();
  if (tid == 0) {
    fenceProxyAsync();
    const uint32_t ub = uint32_t(ecount) * S::USTRIDE * 8, fb = uint32_t(ecount) * S::FSTRIDE * 8;
    mbarExpectTx(bar, a.doVolume ? ub + fb : ub);
    bulkLoad(sU, a.uin + e0 * S::USTRIDE, ub, bar);
    if (a.doVolume) bulkLoad(sF, (a.fluxSrc ? a.fluxSrc : a.face) + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
  }
  if (loadTables)
    if (!GT)
      for (int k = tid; k < int(TAB); k += blockDim.x) tab[k] = tsrc[k];
  __syncthreads();
  const bool arrived = mbarWait(bar, parity);
  if (__syncthreads_or(!arrived)) {
    if (tid == 0) {
      atomicOr(a.status, kStatusTimeout);
      mbarWait(bar, parity);
    }
    return false;
  }
  if (a.doVolume) {
    // values and contravariant fluxes at the volume points
    for (int idx = tid; idx < ecount * NQ; idx += blockDim.x) {
      const int le = idx / NQ, q = idx - le * NQ;
      const int64_t e = e0 + le;
      double U[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) s = fma(phi[q * NB + b], sU[le * S::USTRIDE + v * NB + b], s);
        U[v] = s;
      }
      const double* g = AFFINE ? a.geom + e * GS : a.geom + e * GS + q * GD;
      double ja[DIM][DIM];
#pragma unroll
      for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = 0; c < DIM; ++c) ja[r][c] = g[r * DIM + c];
      State<DIM> st;
      makeState<DIM>(st, U, ph);
      const double ep = energyFluxFactor(st, ph);
      // Boussinesq buoyancy S |J| at the point, kept in the new-state buffer until the residual pass
      if (ph.source) sN[le * NV * NB + q] = st.r * ph.beta * (temperatureOf(st, ph) - ph.tref) / g[DIM * DIM];
      double tau[DIM][DIM] = {}, qh[DIM] = {};
      double avf[VISC == 2 ? NV * DIM : 1];
      if constexpr (VISC != 0) {
        // gradient at the point from the element's modal gradient coefficients [nv*d][NB]
        double g[NV * DIM];
        const double* gc = a.grad + e * NV * DIM * NB;
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) {
          double acc = 0.0;
#pragma unroll
          for (int b = 0; b < NB; ++b) acc = fma(phi[q * NB + b], gc[c * NB + b], acc);
          g[c] = acc;
        }
        if constexpr (VISC == 2) {
          // artificial viscous flux eps(x_q) grad U (ViscousFlux.cpp:105-113), eps from the vertex values
          const double* nod = a.avTab + avDenseNodalOffset(NB, NQ) + q * NF;
          double eps = 0.0;
#pragma unroll
          for (int v = 0; v < NF; ++v) eps = fma(nod[v], a.epsV[e * NF + v], eps);
#pragma unroll
          for (int c = 0; c < NV * DIM; ++c) avf[c] = eps * g[c];
        } else {
          PrimGrad<DIM> pg;
          primitiveGradient<DIM>(g, st.u, st.ir, st.E * st.ir, ph, pg);
          const double u2 = DIM == 2 ? fma(st.u[0], st.u[0], st.u[1] * st.u[1]) : dotn<DIM>(st.u, st.u);
          viscousTensor<DIM>(pg, st.u, fma(ph.incomp ? 0.0 : -0.5, u2, st.E * st.ir) * ph.inv_cv, ph,
                             tau, qh);
        }
      }
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const double vb = dotn<DIM>(st.u, ja[b]);
        double* Q = sQ + ((le * DIM + b) * NV) * NQ + q;
        Q[0] = st.r * vb;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double m = fma(st.m[k], vb, ja[b][k] * st.p);
#pragma unroll
          for (int l = 0; l < DIM; ++l) m = fma(-ja[b][l], tau[l][k], m);
          Q[(1 + k) * NQ] = m;
        }
        Q[(DIM + 1) * NQ] = ep * vb - dotn<DIM>(qh, ja[b]);
        if constexpr (VISC == 2) {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            double x = Q[v * NQ];
#pragma unroll
            for (int l = 0; l < DIM; ++l) x = fma(-ja[b][l], avf[v * DIM + l], x);
            Q[v * NQ] = x;
          }
        }
      }
    }
    __syncthreads();
    // weak residual per basis function
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
        if (ph.source && v == DIM) {  // last momentum component: sum_q w_q |J|_q S_q phi_i(x_q) (affine: M_ref^-1 of it)
          const double* phiw = AFFINE ? tsrc + S::TABLES_AFF
                                      : a.tables + (NQ * NB * (1 + DIM) + NFP * NB * 2 + NB * NB + DIM * NB * NB +
                                                    NF * NB * NFQ + NF * NFQ * NFQ);
          for (int q = 0; q < NQ; ++q) s = fma(sN[le * NV * NB + q], phiw[q * NB + i], s);
        }
        sR[(le * NV + v) * NB + i] = s;
      }
    }
    __syncthreads();
    // du = M^-1 R, RK combination
    for (int idx = tid; idx < ecount * NB; idx += blockDim.x) {
      const int le = idx / NB, i = idx - le * NB;
      const int64_t e = e0 + le;
      const double* g = a.geom + e * GS;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double du;
        if constexpr (AFFINE) {
          du = g[DIM * DIM] * sR[(le * NV + v) * NB + i];  // M^-1 R = (1/|J|) (M_ref^-1 R)
        } else {
          const double* minv = g + NQ * GD;
          double s = 0.0;
          for (int k = 0; k < NB; ++k) s = fma(minv[i * NB + k], sR[(le * NV + v) * NB + k], s);
          du = s;
        }
        sQ[(le * NV + v) * NB + i] = du;  // sQ reused: du per basis function
        if (a.doUpdate) {
          const double u1 = sU[le * S::USTRIDE + v * NB + i];
          // first stage of a step (every RK table starts with {1, 0, 1}): the base state is the staged tile
          const bool first = a.uin == a.ubase && a.c1 == 0.0 && a.c0 == 1.0;
          const double un = first ? fma(a.c2dt, du, u1)
                                  : fma(a.c2dt, du, fma(a.c1, u1, a.c0 * a.ubase[e * S::USTRIDE + v * NB + i]));
          sN[(le * NV + v) * NB + i] = un;
          a.uout[e * S::USTRIDE + v * NB + i] = un;
        } else {
          sN[(le * NV + v) * NB + i] = sU[le * S::USTRIDE + v * NB + i];
        }
      }
    }
    __syncthreads();
    if (a.rate) {
      for (int idx = tid; idx < ecount * NQ; idx += blockDim.x) {
        const int le = idx / NQ, q = idx - le * NQ;
        const int64_t e = e0 + le;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double s = 0.0;
          for (int b = 0; b < NB; ++b) s = fma(phi[q * NB + b], sQ[(le * NV + v) * NB + b], s);
          a.rate[(e * NQ + q) * NV + v] = s;
        }
      }
    }
    if (a.relerr) {
      // relative error: mean over points of |R Phi^T| per element (TimeIntegration.cpp:279-324); affine blocks
      // hold M_ref^-1 R, and R Phi^T = (M_ref^-1 R) (Phi M_ref)^T
      const double* rphi = AFFINE ? mref : phi;
      double acc[NV] = {};
      for (int idx = tid; idx < ecount * NQ; idx += blockDim.x) {
        const int le = idx / NQ, q = idx - le * NQ;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double s = 0.0;
          for (int b = 0; b < NB; ++b) s = fma(rphi[q * NB + b], sR[(le * NV + v) * NB + b], s);
          acc[v] += fabs(s);
        }
      }
      const int warp = tid >> 5, nwarp = blockDim.x >> 5;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double x = acc[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((tid & 31) == 0) sRed[warp * NV + v] = x;
      }
      __syncthreads();
      if (tid < NV) {
        double s = 0.0;
        for (int w = 0; w < nwarp; ++w) s += sRed[w * NV + tid];
        a.relerr[tile * NV + tid] = s / double(NQ);
      }
    }
    __syncthreads();
  } else {
    for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
      const int le = idx / (NV * NB), r = idx - le * NV * NB;
      sN[le * NV * NB + r] = sU[le * S::USTRIDE + r];
    }
    __syncthreads();
  }
  if (a.doTrace) {
    for (int idx = tid; idx < ecount * NFP; idx += blockDim.x) {
      const int le = idx / NFP, fj = idx - le * NFP;
      const int f = fj / NFQ, j = fj - f * NFQ;
      double* out = a.face + (a.faceBase + (e0 + le) * NF + f) * NV * NFQ + j;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double s = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) s = fma(phif[fj * NB + b], sN[(le * NV + v) * NB + b], s);
        out[v * NFQ] = s;
      }
    }
  }
  return true;
}

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int VISC, int DIM = 2>
__global__ void __launch_bounds__(kMaxTileThreads) denseStageKernel(StageArgs a, Phys ph) {
  if (threadIdx.x == 0) mbarInit(denseStageBarrier<NB, NQ, NFQ, NF, AFFINE, DIM>(a.epb), 1);
  denseStageTile<NB, NQ, NFQ, NF, AFFINE, VISC, DIM>(a, ph, blockIdx.x, 0u, true);
}

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int VISC, int DIM = 2>
__global__ void __launch_bounds__(kMaxTileThreads)
    denseStageBatchKernel(const StageArgs* __restrict__ args, const Phys* __restrict__ phys,
                          const int2* __restrict__ items, int nitems, int epb) {
  if (threadIdx.x == 0) mbarInit(denseStageBarrier<NB, NQ, NFQ, NF, AFFINE, DIM>(epb), 1);
  uint32_t parity = 0;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    const StageArgs a = args[it.x];
    const Phys ph = phys[it.x];
    if (!denseStageTile<NB, NQ, NFQ, NF, AFFINE, VISC, DIM>(a, ph, it.y, parity, w == int(blockIdx.x))) return;
    parity ^= 1u;
  }
}


// ---- Navier-Stokes gradient of a dense (modal) block -------------------------------------------------
// R_vg(v*2+k, i) = sum_fj wf_j nF_f[k] X_fj(v) phi_i(x_fj) - sum_q sum_b U_q(v) |J| dxi_b/dx_k w_q dphi_i/dxi_b,
// gradient coefficients = M^-1 R_vg (SpatialDiscrete.cpp:294-322,844-968,1034-1068; TimeIntegration.cpp:200-228).
// X = U+ (neighbour trace) gives the total gradient (BR1, and the BR2 volume-point gradient); X = {U} the BR2
// volume part, to which face f adds its own lift r_f = M^-1 sum_{j in f} wf_j nF_f 1/2[U] phi.
template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
struct DenseGradShape {
  static constexpr int NV = DIM + 2, NFP = NF * NFQ, THREADS = 256;
  static constexpr int USTRIDE = (NV * NB + 1) & ~1;
  static constexpr int FS = NF * NV * NFQ;
  static_assert(AFFINE || DIM == 2, "the general (bilinear) form is built for quadrangles");
  // affine: modal operators (phif, dmod, emod, lmod) and one coefficient block per element;
  // bilinear: the general form with the element's own M^-1
  static constexpr int PER_ELEM = AFFINE ? USTRIDE + 2 * FS + NV * DIM * NB : USTRIDE + 2 * FS + NV * NQ + 3 * NV * 2 * NB;
  static constexpr size_t TABLES = AFFINE ? size_t(NFP) * NB + size_t(DIM) * NB * NB + size_t(NF) * NB * NFQ + size_t(NF) * NFQ * NFQ
                                          : size_t(NQ) * NB * 3 + size_t(NFP) * NB * 2 + size_t(NB) * NB;
  // 8 elements per CTA, fewer where tile and tables would exceed the 227 KB opt-in shared memory (P5
  // tetrahedra: 191 KB of tables, 2 elements)
  static constexpr long long EPB_FIT = (227LL * 1024 - 16 - (long long)TABLES * 8) / ((long long)PER_ELEM * 8);
  static constexpr int EPB = EPB_FIT < 8 ? (EPB_FIT > 0 ? int(EPB_FIT) : 1) : 8;
  static constexpr size_t SMEM = (size_t(EPB) * PER_ELEM + TABLES) * 8 + 16;
  static constexpr size_t smemFor(int epb) { return (size_t(epb) * PER_ELEM + TABLES) * 8 + 16; }
};

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
__device__ __forceinline__ uint64_t* denseGradBarrier(int epb) {
  using G = DenseGradShape<NB, NQ, NFQ, NF, AFFINE, DIM>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  return reinterpret_cast<uint64_t*>(reinterpret_cast<double*>(smem_raw) + epb * G::PER_ELEM + G::TABLES);
}

struct DenseGradArgs {
  const double* u;
  const double* face;
  const double* faceOther;
  double* faceGrad;
  double* grad;             // modal gradient coefficients [e][nv*d][NB]
  const double* geom;
  const double* fmetric;    // [e][NF][d] outward n|J_f|
  const double* tables;
  unsigned* status;
  int64_t ne, faceBase;
  int br2;
  int epb;
  int av;                   // artificial viscosity: grad = the volume-gradient coefficients, traces eps times
                            // the volume-gradient trace, no lifts
  const double* epsV;       // [e][nvert]
  const double* avTab;      // dense artificial-viscosity table
  int fmetricPoint;         // 1: fmetric per face point [e][NF][NFP][d] (curved blocks); 0: per face
  int pad;
};

// Artificial viscosity at face point fj of element e of a dense block (nodal_adjacency_value_ x vertex values).
template <int NB, int NQ, int NVERT>
__device__ __forceinline__ double denseFaceEps(const DenseGradArgs& a, int64_t e, int fj) {
  const double* nf = a.avTab + avDenseNodalFaceOffset(NB, NQ, NVERT) + fj * NVERT;
  double s = 0.0;
#pragma unroll
  for (int v = 0; v < NVERT; ++v) s = fma(nf[v], a.epsV[e * NVERT + v], s);
  return s;
}

// Affine elements: with M = |J| M_ref and constant metric, the gradient coefficients are
//   w_tot(v,k) = (1/|J|) [ sum_f nF_f[k] E_f U+_f(v) - sum_b |J| dxi_b/dx_k D_b u(v) ]
//   w_vol(v,k) = w_tot(v,k) - (1/|J|) sum_f nF_f[k] E_f (1/2 [U])_f(v)
// and the BR2 trace at face f adds (1/|J|) nF_f L_f (1/2 [U])_f: the same quantities as the general form
// below, with M^-1 folded into the precomputed operators.
template <int NB, int NQ, int NFQ, int NF, int DIM = 2>
__device__ __forceinline__ bool denseGradientAffineTile(const DenseGradArgs& a, int64_t tile, uint32_t parity,
                                                        bool loadTables) {
  using G = DenseGradShape<NB, NQ, NFQ, NF, true, DIM>;
  constexpr int NV = DIM + 2, NFP = G::NFP, FS = G::FS, NR = NV * DIM, GD = DIM * DIM + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int EPB = a.epb;
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE] modal coefficients
  double* sS = sU + EPB * G::USTRIDE;                // own traces [EPB][FS]
  double* sO = sS + EPB * FS;                        // other traces [EPB][FS]
  double* sW = sO + EPB * FS;                        // coefficients whose traces are the face gradients [EPB][NR][NB]
  double* tab = sW + EPB * NR * NB;
  const double* phif = tab;                          // [NFP][NB]
  const double* dmod = phif + NFP * NB;              // [DIM][NB][NB]
  const double* emod = dmod + DIM * NB * NB;         // [NF][NB][NFQ]
  const double* lmod = emod + NF * NB * NFQ;         // [NF][NFQ][NFQ]
  uint64_t* bar = reinterpret_cast<uint64_t*>(tab + G::TABLES);

  const int tid = threadIdx.x;
  const int64_t e0 = tile * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  __syncthreads();
  if (tid == 0) {
    fenceProxyAsync();
    const uint32_t ub = uint32_t(ecount) * G::USTRIDE * 8, fb = uint32_t(ecount) * FS * 8;
    mbarExpectTx(bar, ub + 2 * fb);
    bulkLoad(sU, a.u + e0 * G::USTRIDE, ub, bar);
    bulkLoad(sS, a.face + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
    bulkLoad(sO, a.faceOther + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
  }
  if (loadTables) {
    constexpr int OFF_PHIF = NQ * NB * (1 + DIM), OFF_DMOD = NQ * NB * (1 + DIM) + NFP * NB * 2 + NB * NB;
    constexpr int NOPS = DIM * NB * NB + NF * NB * NFQ + NF * NFQ * NFQ;
    for (int k = tid; k < NFP * NB; k += blockDim.x) tab[k] = a.tables[OFF_PHIF + k];
    for (int k = tid; k < NOPS; k += blockDim.x) tab[NFP * NB + k] = a.tables[OFF_DMOD + k];
  }
  __syncthreads();
  const bool arrived = mbarWait(bar, parity);
  if (__syncthreads_or(!arrived)) {
    if (tid == 0) {
      atomicOr(a.status, kStatusTimeout);
      mbarWait(bar, parity);
    }
    return false;
  }
  // 0. the own traces are only needed through the jump 1/2 (U+ - U-): form it once per face point
  for (int k = tid; k < ecount * FS; k += blockDim.x) sS[k] = 0.5 * (sO[k] - sS[k]);
  __syncthreads();
  // 1. coefficients per (element, variable, basis function)
  for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
    const int le = idx / (NV * NB), r = idx - le * NV * NB;
    const int v = r / NB, i = r - v * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GD;
    const double jinv = g[DIM * DIM];
    const double* u = sU + le * G::USTRIDE + v * NB;
    double d[DIM] = {};
#pragma unroll
    for (int m = 0; m < NB; ++m) {
#pragma unroll
      for (int b = 0; b < DIM; ++b) d[b] = fma(dmod[(b * NB + i) * NB + m], u[m], d[b]);
    }
    // tot_k = -sum_b (|J| dxi_b/dx_k) d_b, jmp_k: the BR2 jump part
    double tot[DIM], jmp[DIM] = {};
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      double s = g[(DIM - 1) * DIM + k] * d[DIM - 1];
#pragma unroll
      for (int b = DIM - 2; b >= 0; --b) s = fma(g[b * DIM + k], d[b], s);
      tot[k] = -s;
    }
    const double* nF = a.fmetric + e * NF * DIM;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const double* O = sO + le * FS + (f * NV + v) * NFQ;
      const double* Jm = sS + le * FS + (f * NV + v) * NFQ;  // 1/2 (U+ - U-)
      const double* E = emod + (f * NB + i) * NFQ;
      double ep = 0.0, ej = 0.0;
#pragma unroll
      for (int j = 0; j < NFQ; ++j) {
        ep = fma(E[j], O[j], ep);
        ej = fma(E[j], Jm[j], ej);
      }
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        tot[k] = fma(nF[f * DIM + k], ep, tot[k]);
        jmp[k] = fma(nF[f * DIM + k], ej, jmp[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      const double gk = jinv * tot[k];
      // artificial viscosity keeps the volume-gradient coefficients (ViscousFluxEnum::None gradient)
      a.grad[(e * NR + v * DIM + k) * NB + i] = a.av ? jinv * (tot[k] - jmp[k]) : gk;
      sW[(le * NR + v * DIM + k) * NB + i] = a.br2 ? jinv * (tot[k] - jmp[k]) : gk;
    }
  }
  __syncthreads();
  // 2. face gradient traces per (element, face point, variable)
  for (int idx = tid; idx < ecount * NFP * NV; idx += blockDim.x) {
    const int le = idx / (NFP * NV), r = idx - le * NFP * NV;
    const int fj = r / NV, v = r - fj * NV;
    const int f = fj / NFQ, j = fj - f * NFQ;
    const int64_t e = e0 + le;
    const double* w = sW + (le * NR + v * DIM) * NB;
    double acc[DIM] = {};
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
      for (int k = 0; k < DIM; ++k) acc[k] = fma(phif[fj * NB + b], w[k * NB + b], acc[k]);
    }
    if (a.av) {
      const double eps = denseFaceEps<NB, NQ, NF>(a, e, fj);
#pragma unroll
      for (int k = 0; k < DIM; ++k) acc[k] *= eps;
    } else if (a.br2) {
      const double* Jm = sS + le * FS + (f * NV + v) * NFQ;
      const double* L = lmod + (f * NFQ + j) * NFQ;
      double lift = 0.0;
#pragma unroll
      for (int jj = 0; jj < NFQ; ++jj) lift = fma(L[jj], Jm[jj], lift);
      lift *= a.geom[e * GD + DIM * DIM];
#pragma unroll
      for (int k = 0; k < DIM; ++k) acc[k] = fma(a.fmetric[(e * NF + f) * DIM + k], lift, acc[k]);
    }
    double* out = a.faceGrad + (a.faceBase + e * NF + f) * NR * NFQ + j;
#pragma unroll
    for (int k = 0; k < DIM; ++k) out[(v * DIM + k) * NFQ] = acc[k];
  }
  return true;
}

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
__device__ __forceinline__ bool denseGradientTile(const DenseGradArgs& a, int64_t tile, uint32_t parity, bool loadTables) {
  if constexpr (AFFINE) return denseGradientAffineTile<NB, NQ, NFQ, NF, DIM>(a, tile, parity, loadTables);
  using G = DenseGradShape<NB, NQ, NFQ, NF, AFFINE>;
  constexpr int NV = 4, NFP = G::NFP, FS = G::FS, NR = NV * 2;
  const int EPB = a.epb;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sU = reinterpret_cast<double*>(smem_raw);  // [EPB][USTRIDE] modal coefficients
  double* sS = sU + EPB * G::USTRIDE;                // own traces [EPB][FS]
  double* sO = sS + EPB * FS;                        // other traces [EPB][FS]
  double* sUq = sO + EPB * FS;                       // values at the volume points [EPB][NV][NQ]
  double* sRt = sUq + EPB * NV * NQ;                 // total gradient residual / coefficients [EPB][NR][NB]
  double* sRv = sRt + EPB * NR * NB;                 // BR2 volume part [EPB][NR][NB]
  double* sRf = sRv + EPB * NR * NB;                 // BR2 face-lift residual of one face [EPB][NR][NB]
  double* tab = sRf + EPB * NR * NB;
  const double* phi = tab;
  const double* dphiw = phi + NQ * NB;
  const double* phif = dphiw + NQ * 2 * NB;
  const double* phifw = phif + NFP * NB;
  const double* mref = phifw + NFP * NB;
  uint64_t* bar = reinterpret_cast<uint64_t*>(tab + G::TABLES);
  const int GS = AFFINE ? 5 : NQ * 5 + NB * NB;

  const int tid = threadIdx.x;
  const int64_t e0 = tile * EPB;
  const int ecount = int(a.ne - e0 < EPB ? a.ne - e0 : EPB);
  __syncthreads();
  if (tid == 0) {
    fenceProxyAsync();
    const uint32_t ub = uint32_t(ecount) * G::USTRIDE * 8, fb = uint32_t(ecount) * FS * 8;
    mbarExpectTx(bar, ub + 2 * fb);
    bulkLoad(sU, a.u + e0 * G::USTRIDE, ub, bar);
    bulkLoad(sS, a.face + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
    bulkLoad(sO, a.faceOther + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
  }
  if (loadTables)
    for (int k = tid; k < int(G::TABLES); k += blockDim.x) tab[k] = a.tables[k];
  __syncthreads();
  const bool arrived = mbarWait(bar, parity);
  if (__syncthreads_or(!arrived)) {
    if (tid == 0) {
      atomicOr(a.status, kStatusTimeout);
      mbarWait(bar, parity);
    }
    return false;
  }
  // values at the volume points; the own traces are only needed through {U} = 1/2 (U+ + U-) (volume part)
  // and 1/2 [U] = U+ - {U} (lifts): the average replaces them, once per face point
  for (int idx = tid; idx < ecount * NV * NQ; idx += blockDim.x) {
    const int le = idx / (NV * NQ), r = idx - le * NV * NQ;
    const int v = r / NQ, q = r - v * NQ;
    double acc = 0.0;
#pragma unroll
    for (int b = 0; b < NB; ++b) acc = fma(phi[q * NB + b], sU[le * G::USTRIDE + v * NB + b], acc);
    sUq[(le * NV + v) * NQ + q] = acc;
  }
  for (int k = tid; k < ecount * FS; k += blockDim.x) sS[k] = 0.5 * (sO[k] + sS[k]);
  __syncthreads();
  // gradient residuals (total, BR2 volume part)
  for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
    const int le = idx / (NV * NB), r = idx - le * NV * NB;
    const int v = r / NB, i = r - v * NB;
    const int64_t e = e0 + le;
    double tot[2] = {0.0, 0.0}, vol[2] = {0.0, 0.0};
    for (int fj = 0; fj < NFP; ++fj) {
      const int f = fj / NFQ, j = fj - f * NFQ;
      // outward n|J_f| of face f (per face point on curved blocks)
      const double* nF = a.fmetric + (a.fmetricPoint ? (e * NF + f) * NFQ + j : e * NF + f) * 2;
      const double w = phifw[fj * NB + i];
      const double o = sO[le * FS + (f * NV + v) * NFQ + j], avg = sS[le * FS + (f * NV + v) * NFQ + j];
      const double xt = w * o, xv = w * avg;
      tot[0] = fma(xt, nF[0], tot[0]); tot[1] = fma(xt, nF[1], tot[1]);
      vol[0] = fma(xv, nF[0], vol[0]); vol[1] = fma(xv, nF[1], vol[1]);
    }
    double d[2][2] = {{0.0, 0.0}, {0.0, 0.0}};  // d[b][k] = sum_q U_q |J| dxi_b/dx_k w_q dphi_i/dxi_b
    for (int q = 0; q < NQ; ++q) {
      const double uq = sUq[(le * NV + v) * NQ + q];
      const double* g = AFFINE ? a.geom + e * GS : a.geom + e * GS + q * 5;
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const double t = uq * dphiw[(q * 2 + b) * NB + i];
        d[b][0] = fma(t, g[b * 2 + 0], d[b][0]);
        d[b][1] = fma(t, g[b * 2 + 1], d[b][1]);
      }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      sRt[(le * NR + v * 2 + k) * NB + i] = tot[k] - d[0][k] - d[1][k];
      sRv[(le * NR + v * 2 + k) * NB + i] = vol[k] - d[0][k] - d[1][k];
    }
  }
  __syncthreads();
  // M^-1 (affine: M_ref^-1 / |J|; bilinear: the element's inverse); total coefficients -> global
  for (int idx = tid; idx < ecount * NR * NB; idx += blockDim.x) {
    const int le = idx / (NR * NB), r = idx - le * NR * NB;
    const int c = r / NB, i = r - c * NB;
    const int64_t e = e0 + le;
    const double* g = a.geom + e * GS;
    const double* minv = AFFINE ? mref : g + NQ * 5;
    const double sc = AFFINE ? g[4] : 1.0;
    double t = 0.0, w = 0.0;
    for (int k = 0; k < NB; ++k) {
      t = fma(minv[i * NB + k], sRt[(le * NR + c) * NB + k], t);
      w = fma(minv[i * NB + k], sRv[(le * NR + c) * NB + k], w);
    }
    a.grad[(e * NR + c) * NB + i] = a.av ? sc * w : sc * t;
    sRf[(le * NR + c) * NB + i] = sc * w;  // staged: BR2 volume coefficients
  }
  __syncthreads();
  for (int idx = tid; idx < ecount * NR * NB; idx += blockDim.x) {
    const int le = idx / (NR * NB), r = idx - le * NR * NB;
    sRv[le * NR * NB + r] = sRf[le * NR * NB + r];
    if (!a.br2) sRt[le * NR * NB + r] = a.grad[((e0 + le) * NR) * NB + r];
  }
  __syncthreads();
  if (!a.br2 || a.av) {
    // BR1 face gradient traces: trace of the total gradient; artificial viscosity: eps times the trace of
    // the volume gradient
    const double* src = a.av ? sRv : sRt;
    for (int idx = tid; idx < ecount * NFP; idx += blockDim.x) {
      const int le = idx / NFP, fj = idx - le * NFP;
      const int f = fj / NFQ, j = fj - f * NFQ;
      double* out = a.faceGrad + (a.faceBase + (e0 + le) * NF + f) * NR * NFQ + j;
      const double eps = a.av ? denseFaceEps<NB, NQ, NF>(a, e0 + le, fj) : 1.0;
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) acc = fma(phif[fj * NB + b], src[(le * NR + c) * NB + b], acc);
        out[c * NFQ] = eps * acc;
      }
    }
    return true;
  }
  // BR2: for each face f, trace of (volume gradient + r_f), r_f = M^-1 sum_{j in f} wf_j nF_f 1/2[U] phi
  for (int f = 0; f < NF; ++f) {
    for (int idx = tid; idx < ecount * NV * NB; idx += blockDim.x) {
      const int le = idx / (NV * NB), r = idx - le * NV * NB;
      const int v = r / NB, i = r - v * NB;
      double acc0 = 0.0, acc1 = 0.0;
      if (a.fmetricPoint) {  // curved: n|J_f| varies along the face
        for (int j = 0; j < NFQ; ++j) {
          const double* nF = a.fmetric + (((e0 + le) * NF + f) * NFQ + j) * 2;
          const double jump = sO[le * FS + (f * NV + v) * NFQ + j] - sS[le * FS + (f * NV + v) * NFQ + j];
          const double t = phifw[(f * NFQ + j) * NB + i] * jump;
          acc0 = fma(t, nF[0], acc0);
          acc1 = fma(t, nF[1], acc1);
        }
      } else {
        const double* nF = a.fmetric + (e0 + le) * NF * 2 + f * 2;
        double acc = 0.0;
        for (int j = 0; j < NFQ; ++j) {
          const double jump = sO[le * FS + (f * NV + v) * NFQ + j] - sS[le * FS + (f * NV + v) * NFQ + j];
          acc = fma(phifw[(f * NFQ + j) * NB + i], jump, acc);
        }
        acc0 = acc * nF[0];
        acc1 = acc * nF[1];
      }
      sRt[(le * NR + v * 2 + 0) * NB + i] = acc0;
      sRt[(le * NR + v * 2 + 1) * NB + i] = acc1;
    }
    __syncthreads();
    for (int idx = tid; idx < ecount * NR * NB; idx += blockDim.x) {
      const int le = idx / (NR * NB), r = idx - le * NR * NB;
      const int c = r / NB, i = r - c * NB;
      const int64_t e = e0 + le;
      const double* g = a.geom + e * GS;
      const double* minv = AFFINE ? mref : g + NQ * 5;
      const double sc = AFFINE ? g[4] : 1.0;
      double t = 0.0;
      for (int k = 0; k < NB; ++k) t = fma(minv[i * NB + k], sRt[(le * NR + c) * NB + k], t);
      sRf[(le * NR + c) * NB + i] = sRv[(le * NR + c) * NB + i] + sc * t;
    }
    __syncthreads();
    for (int idx = tid; idx < ecount * NFQ; idx += blockDim.x) {
      const int le = idx / NFQ, j = idx - le * NFQ;
      const int fj = f * NFQ + j;
      double* out = a.faceGrad + (a.faceBase + (e0 + le) * NF + f) * NR * NFQ + j;
#pragma unroll
      for (int c = 0; c < NR; ++c) {
        double acc = 0.0;
#pragma unroll
        for (int b = 0; b < NB; ++b) acc = fma(phif[fj * NB + b], sRf[(le * NR + c) * NB + b], acc);
        out[c * NFQ] = acc;
      }
    }
    __syncthreads();
  }
  return true;
}

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
__global__ void __launch_bounds__(kMaxTileThreads) denseGradientKernel(DenseGradArgs a) {
  if (threadIdx.x == 0) mbarInit(denseGradBarrier<NB, NQ, NFQ, NF, AFFINE, DIM>(a.epb), 1);
  denseGradientTile<NB, NQ, NFQ, NF, AFFINE, DIM>(a, blockIdx.x, 0u, true);
}

template <int NB, int NQ, int NFQ, int NF, bool AFFINE, int DIM = 2>
__global__ void __launch_bounds__(kMaxTileThreads)
    denseGradientBatchKernel(const DenseGradArgs* __restrict__ args, const int2* __restrict__ items, int nitems, int epb) {
  if (threadIdx.x == 0) mbarInit(denseGradBarrier<NB, NQ, NFQ, NF, AFFINE, DIM>(epb), 1);
  uint32_t parity = 0;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    const DenseGradArgs a = args[it.x];
    if (!denseGradientTile<NB, NQ, NFQ, NF, AFFINE, DIM>(a, it.y, parity, w == int(blockIdx.x))) return;
    parity ^= 1u;
  }
}

// Tetrahedra (dense blocks of DIM 3, affine): P = 1..3 with the Keast rules of 4, 11, 24 points and the
// Dunavant face rules of 4, 7, 13 points.
#define SDG_TET_ADJOINT_CASES(X)                \
  X(SDG_ELEMENT_TETRAHEDRON, 1, 4, 4, 4, 4)     \
  X(SDG_ELEMENT_TETRAHEDRON, 2, 10, 11, 7, 4)   \
  X(SDG_ELEMENT_TETRAHEDRON, 3, 20, 24, 13, 4)
// P4: 35 modes, the 69-point Grundmann-Moeller volume rule (tetrahedron_rules.h), 19-point faces; P5: 56 modes,
// the 125-point Grundmann-Moeller rule, 27-point faces, the stage tables read from global memory.  Stage and
// gradient kernels only (the derivative kernels' tables would not fit the shared memory)
#define SDG_TET_CASES(X)                        \
  SDG_TET_ADJOINT_CASES(X)                      \
  X(SDG_ELEMENT_TETRAHEDRON, 4, 35, 69, 19, 4)  \
  X(SDG_ELEMENT_TETRAHEDRON, 5, 56, 125, 27, 4)

// (type, P) -> (NB, NQ, NFQ): triangle P1..P5 use Dunavant rules of 3,6,12,16,25 points.

// The element blocks with derivative kernels (every dense block of 2D, curved triangles included).
#define SDG_DENSE_ADJOINT_CASES(X)                          \
  X(SDG_ELEMENT_TRIANGLE, 1, 3, 3, 2, 3, true)              \
  X(SDG_ELEMENT_TRIANGLE, 2, 6, 6, 3, 3, true)              \
  X(SDG_ELEMENT_TRIANGLE, 3, 10, 12, 4, 3, true)            \
  X(SDG_ELEMENT_TRIANGLE, 4, 15, 16, 5, 3, true)            \
  X(SDG_ELEMENT_TRIANGLE, 5, 21, 25, 6, 3, true)            \
  X(SDG_ELEMENT_QUADRANGLE, 1, 4, 7, 2, 4, true)            \
  X(SDG_ELEMENT_QUADRANGLE, 1, 4, 7, 2, 4, false)           \
  X(SDG_ELEMENT_TRIANGLE, 1, 3, 3, 2, 3, false)             \
  X(SDG_ELEMENT_TRIANGLE, 2, 6, 6, 3, 3, false)             \
  X(SDG_ELEMENT_TRIANGLE, 3, 10, 12, 4, 3, false)           \
  X(SDG_ELEMENT_TRIANGLE, 4, 15, 16, 5, 3, false)           \
  X(SDG_ELEMENT_TRIANGLE, 5, 21, 25, 6, 3, false)

// Forward kernels: the same blocks.
#define SDG_DENSE_CASES(X)                                  \
  X(SDG_ELEMENT_TRIANGLE, 1, 3, 3, 2, 3, true)              \
  X(SDG_ELEMENT_TRIANGLE, 2, 6, 6, 3, 3, true)              \
  X(SDG_ELEMENT_TRIANGLE, 3, 10, 12, 4, 3, true)            \
  X(SDG_ELEMENT_TRIANGLE, 4, 15, 16, 5, 3, true)            \
  X(SDG_ELEMENT_TRIANGLE, 5, 21, 25, 6, 3, true)            \
  X(SDG_ELEMENT_TRIANGLE, 1, 3, 3, 2, 3, false)             \
  X(SDG_ELEMENT_TRIANGLE, 2, 6, 6, 3, 3, false)             \
  X(SDG_ELEMENT_TRIANGLE, 3, 10, 12, 4, 3, false)           \
  X(SDG_ELEMENT_TRIANGLE, 4, 15, 16, 5, 3, false)           \
  X(SDG_ELEMENT_TRIANGLE, 5, 21, 25, 6, 3, false)           \
  X(SDG_ELEMENT_QUADRANGLE, 1, 4, 7, 2, 4, true)            \
  X(SDG_ELEMENT_QUADRANGLE, 1, 4, 7, 2, 4, false)

}  // namespace sdg
