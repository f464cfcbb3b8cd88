// Navier-Stokes (BR1/BR2) kernels of the GB300 DG path: trace exchange, weak gradient, viscous face flux.
//
// Per RK stage the reference runs the gradient pass (src/Solver/TimeIntegration.cpp:340-343):
//   volume gradient quadrature      SpatialDiscrete.cpp:294-322
//   face gradient fluxes            SpatialDiscrete.cpp:844-968  ({U} n |J_f| w, and 1/2 [U] n |J_f| w)
//   gradient residual + M^-1        SpatialDiscrete.cpp:1034-1068, TimeIntegration.cpp:200-228
// then the viscous volume flux (SpatialDiscrete.cpp:194-266) and the central viscous face flux
// (SpatialDiscrete.cpp:633-842, ViscousFlux.cpp:138-170).
//
// With the nodal Gauss basis the gradient of conserved variable v, component k, at node i is
//   w_k(i) = (1/|J|_i) [ sum_f Lhat_e(i_b) nF_f[k] X_f(j) - sum_b sum_a Dhat(a, i_b) (U |J| dxi_b/dx_k)(a) ]
// with X = the neighbour trace U+ for the total gradient (the BR1 gradient, and the BR2 volume gradient:
// {U} + 1/2 [U] = U+), X = {U} for the BR2 "volume" part.  nF_f = n |J_f| of face f; for affine elements
// Nanson's relation gives nF_f = +-|J| dxi_b/dx (the metric row of the face's axis).  BR2 face gradients add
// the face's own lift r_f, whose trace at its face is nF_f 1/2[U] sum_a l_a(end)^2 / (w_a |J|_a).
//
// Face buffers (NS): face = own traces, faceOther = neighbour traces (exchange kernel),
// faceGrad = gradient traces [slot][v*d+k][j], faceFlux = outward |J_f| (h - h_visc) per slot.
#pragma once
#include "sdg_kernels.cuh"

namespace sdg {

struct GradArgs {
  const double* u;          // state [e][USTRIDE]
  const double* face;       // own traces
  const double* faceOther;  // neighbour traces
  double* faceGrad;         // gradient traces out, slot stride d*nv*nfq
  double* grad;             // total gradient at the nodes out, [e][nv*d][NB]
  const double* geom;       // as the stage kernel
  const double* fmetric;    // bilinear blocks: [e][nface][d] outward n|J_f|; null for affine
  const double* tables;
  unsigned* status;
  int64_t ne, faceBase;
  int br2;
  int epb;                  // elements per CTA tile
  int av;                   // artificial viscosity (BR2 layout): grad = eps times the volume gradient, traces
                            // eps times the volume-gradient trace, no lifts
  const double* epsV;       // [e][nvert] artificial viscosity at the vertices
  const double* avTab;      // tensor artificial-viscosity table (x[N] first)
  int fmetricPoint;         // 1: fmetric per face point [e][nface][nfq][d] (curved blocks); 0: per face
  int pad;
};

// Exchange of traces across interior faces: each side receives the other side's trace at its own points.
template <int DIM>
__device__ __forceinline__ void exchangePoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = a.face[L + v * nfq], y = a.face[R + v * nfq];
    a.other[L + v * nfq] = y;
    a.other[R + v * nfq] = x;
  }
}

// Boundary neighbour trace for the gradient: 2 U_b - U, where U_b is the boundary's gradient state
// (BoundaryCondition.cpp: U for farfield/inflow/outflow, the wall state for walls); then {U} = U_b and
// the interface jump 1/2 (U+ - U) = U_b - U, as the reference's boundary gradient fluxes.
template <int DIM>
__device__ __forceinline__ void exchangeBoundaryPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j;
  double ul[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = a.face[L + v * nfq];
  if (bc <= 2) {
#pragma unroll
    for (int v = 0; v < NV; ++v) a.other[L + v * nfq] = ul[v];
    return;
  }
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  State<DIM> s;
  makeState<DIM>(s, ul, a.ph);
  Comp<DIM> l, g, b;
  compFromState<DIM>(s, l, a.ph);
  const double* gp = a.ghost + (f * nfq + j) * (DIM + 3);
  g.r = gp[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gp[1 + k];
  g.e = gp[DIM + 1];
  g.p = gp[DIM + 2];
  boundaryState<DIM>(bc, n, l, g, a.ph, b);
  double ub[NV];
  ub[0] = b.r;
#pragma unroll
  for (int k = 0; k < DIM; ++k) ub[1 + k] = b.r * b.u[k];
  ub[DIM + 1] = energyOfComp<DIM>(b, a.ph);
#pragma unroll
  for (int v = 0; v < NV; ++v) a.other[L + v * nfq] = 2.0 * ub[v] - ul[v];
}

// First-order nodal (vertex) basis of a line / quadrangle / hexahedron at reference point X (gmsh vertex
// order: -1, 1; (-1,-1), (1,-1), (1,1), (-1,1), then the same at z = +1), the artificial viscosity's
// interpolation (BasisFunction.cpp:200-208 nodal_value_).
template <int DIM>
__device__ __forceinline__ double vertexWeight(int v, const double* X) {
  if constexpr (DIM == 1) return 0.5 * (1.0 + (v == 1 ? 1.0 : -1.0) * X[0]);
  const double sx = (v & 3) == 1 || (v & 3) == 2 ? 1.0 : -1.0;
  const double sy = (v & 3) >= 2 ? 1.0 : -1.0;
  double w = 0.25 * (1.0 + sx * X[0]) * (1.0 + sy * X[1]);
  if constexpr (DIM == 3) w *= 0.5 * (1.0 + (v >= 4 ? 1.0 : -1.0) * X[2]);
  return w;
}

template <int DIM>
__device__ __forceinline__ double vertexInterp(const double* epsV, const double* X) {
  constexpr int NVERT = 1 << DIM;
  double s = 0.0;
#pragma unroll
  for (int v = 0; v < NVERT; ++v) s = fma(vertexWeight<DIM>(v, X), epsV[v], s);
  return s;
}

template <int DIM, int N, bool AFFINE, bool BR2>
struct GradShape {
  using S = TensorShape<DIM, N>;
  static constexpr int NV = S::NV, NB = S::NB, NF = S::NF, NFQ = S::NFQ;
  static constexpr int FS = NF * NV * NFQ;      // trace slots per element (one area)
  static constexpr int GSTR = NV * DIM * NB;    // gradient doubles per element
  static constexpr int PSZ = AFFINE ? 0 : DIM * DIM * NV * NB;  // bilinear: U |J| dxi_b/dx_k per node
  // shared memory per element: state, own traces, other traces, gradient (total; BR2 also the volume
  // gradient), metric products (bilinear), 1/|J|
  static constexpr int PER_ELEM = S::USTRIDE + (BR2 ? 2 : 1) * FS + (BR2 ? 2 : 1) * GSTR + PSZ + NB;
  static constexpr int EPB_SMEM = (100 * 1024) / (8 * PER_ELEM) > 0 ? (100 * 1024) / (8 * PER_ELEM) : 1;
  static constexpr int EPB = S::EPB_RAW < EPB_SMEM ? S::EPB_RAW : EPB_SMEM;
  static constexpr int THREADS = ((EPB * NB + 31) / 32) * 32;
  static constexpr size_t SMEM = size_t(EPB) * PER_ELEM * 8 + sizeof(TensorTables) + 16;
  static constexpr int threadsFor(int epb) { return ((epb * NB + 31) / 32) * 32; }
  static constexpr size_t smemFor(int epb) { return size_t(epb) * PER_ELEM * 8 + sizeof(TensorTables) + 16; }
};

template <int DIM, int N, bool AFFINE, bool BR2>
__device__ __forceinline__ uint64_t* tensorGradBarrier(int epb) {
  using G = GradShape<DIM, N, AFFINE, BR2>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* end = reinterpret_cast<double*>(smem_raw) + epb * G::PER_ELEM;
  return reinterpret_cast<uint64_t*>(reinterpret_cast<TensorTables*>(end) + 1);
}

// Weak (BR) gradient of a tensor block, one tile: one thread per node.  Writes the total gradient at the
// nodes and the face gradient traces (BR1: total gradient; BR2: volume gradient + the face's own lift).
template <int DIM, int N, bool AFFINE, bool BR2>
__device__ __forceinline__ bool tensorGradientTile(const GradArgs& a, int64_t tile, uint32_t parity, bool loadTables) {
  using G = GradShape<DIM, N, AFFINE, BR2>;
  using S = TensorShape<DIM, N>;
  constexpr int NV = G::NV, NB = G::NB, NF = G::NF, NFQ = G::NFQ, FS = G::FS;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int epb = a.epb;
  double* sU = reinterpret_cast<double*>(smem_raw);  // [epb][USTRIDE]
  double* sS = sU + epb * S::USTRIDE;                // own traces [epb][FS] (BR2 only)
  double* sO = sS + (BR2 ? epb * FS : 0);            // other traces [epb][FS]
  double* sGt = sO + epb * FS;                       // total gradient [epb][NV*DIM][NB]
  double* sGv = sGt + (BR2 ? epb * G::GSTR : 0);    // BR2 volume gradient [epb][NV*DIM][NB]
  double* sP = sGv + epb * G::GSTR;                  // bilinear: U |J| dxi_b/dx_k [epb][DIM*DIM*NV][NB]
  double* sJ = sP + epb * G::PSZ;                    // 1/|J| per node [epb][NB]
  TensorTables* T = reinterpret_cast<TensorTables*>(sJ + epb * NB);
  uint64_t* bar = reinterpret_cast<uint64_t*>(T + 1);

  const int tid = threadIdx.x;
  const int64_t e0 = tile * epb;
  const int ecount = int(a.ne - e0 < epb ? a.ne - e0 : epb);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;
  __syncthreads();
  if (tid == 0) {
    fenceProxyAsync();
    const uint32_t ub = uint32_t(ecount) * S::USTRIDE * 8, fb = uint32_t(ecount) * FS * 8;
    mbarExpectTx(bar, ub + (BR2 ? 2 : 1) * fb);
    bulkLoad(sU, a.u + e0 * S::USTRIDE, ub, bar);
    if (BR2) bulkLoad(sS, a.face + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
    bulkLoad(sO, a.faceOther + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
  }
  if (loadTables)
    for (int k = tid; k < int(sizeof(TensorTables) / 8); k += blockDim.x) reinterpret_cast<double*>(T)[k] = a.tables[k];
  __syncthreads();
  const bool arrived = mbarWait(bar, parity);
  if (__syncthreads_or(!arrived)) {
    if (tid == 0) {
      atomicOr(a.status, kStatusTimeout);
      mbarWait(bar, parity);
    }
    return false;
  }
  constexpr int GS = DIM * DIM + 1;
  // BR2: the own traces are only needed through {U} = 1/2 (U+ + U-) (volume gradient) and 1/2 [U] = U+ - {U}
  // (lift): form the average once per face point instead of once per node on its line
  if constexpr (BR2) {
    for (int k = tid; k < ecount * FS; k += blockDim.x) sS[k] = 0.5 * (sO[k] + sS[k]);
  }
  int ax[DIM];
#pragma unroll
  for (int b = 0; b < DIM; ++b) ax[b] = axisIndex<DIM, N>(node, b);
  double jinv = 0.0, ja[DIM][DIM];
  if (active) {
    const double* g = AFFINE ? a.geom + e * GS : a.geom + (e * NB + node) * GS;
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
    jinv = g[DIM * DIM];
    sJ[le * NB + node] = jinv;
    if constexpr (!AFFINE) {
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const double u = sU[le * S::USTRIDE + v * NB + node];
#pragma unroll
        for (int b = 0; b < DIM; ++b)
#pragma unroll
          for (int k = 0; k < DIM; ++k) sP[((le * DIM + b) * DIM + k) * NV * NB + v * NB + node] = u * ja[b][k];
      }
    }
  }
  __syncthreads();
  double epsNode = 0.0;
  if constexpr (BR2) {
    if (a.av && active) {
      double X[DIM];
#pragma unroll
      for (int b = 0; b < DIM; ++b) X[b] = a.avTab[ax[b]];
      epsNode = vertexInterp<DIM>(a.epsV + e * (1 << DIM), X);
    }
  }
  if (active) {
    double nF[DIM][2][DIM];  // outward n|J_f| of the faces (axis b, end)
#pragma unroll
    for (int b = 0; b < DIM; ++b)
#pragma unroll
      for (int en = 0; en < 2; ++en)
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          if constexpr (AFFINE) nF[b][en][k] = en ? ja[b][k] : -ja[b][k];
          else if (a.fmetricPoint)
            nF[b][en][k] = a.fmetric[((e * NF + T->axisFace[b][en]) * NFQ + T->nodeFacePoint[b][en][node]) * DIM + k];
          else nF[b][en][k] = a.fmetric[(e * NF + T->axisFace[b][en]) * DIM + k];
        }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double tot[DIM], vol[DIM], dsum[DIM];  // dsum (non-affine): -sum_b of the line derivatives, added once
#pragma unroll
      for (int k = 0; k < DIM; ++k) { tot[k] = 0.0; vol[k] = 0.0; dsum[k] = 0.0; }
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const int st = strideOf<DIM, N>(b);
        const int base = node - ax[b] * st;
        const double lm = T->liftm[ax[b]], lp = T->liftp[ax[b]];
        const int fm = T->axisFace[b][0], fp = T->axisFace[b][1];
        const int jm = T->nodeFacePoint[b][0][node], jp = T->nodeFacePoint[b][1][node];
        const double om = sO[le * FS + (fm * NV + v) * NFQ + jm], op = sO[le * FS + (fp * NV + v) * NFQ + jp];
        const double am = BR2 ? sS[le * FS + (fm * NV + v) * NFQ + jm] : 0.0;  // {U} at the two ends
        const double ap = BR2 ? sS[le * FS + (fp * NV + v) * NFQ + jp] : 0.0;
        if constexpr (AFFINE) {
          double dref = 0.0;
#pragma unroll
          for (int q = 0; q < N; ++q) dref = fma(T->dhat[q][ax[b]], sU[le * S::USTRIDE + v * NB + base + q * st], dref);
          // |J| dxi_b/dx_k . (Lhat+ X+ - Lhat- X- - dref); nF(b,+) = -nF(b,-) = |J| dxi_b/dx
          const double tt = fma(lp, op, fma(-lm, om, -dref));
#pragma unroll
          for (int k = 0; k < DIM; ++k) tot[k] = fma(ja[b][k], tt, tot[k]);
          if constexpr (BR2) {
            const double tv = fma(lp, ap, fma(-lm, am, -dref));
#pragma unroll
            for (int k = 0; k < DIM; ++k) vol[k] = fma(ja[b][k], tv, vol[k]);
          }
        } else {
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            double dk = dsum[k];
            const double* P = sP + ((le * DIM + b) * DIM + k) * NV * NB + v * NB + base;
#pragma unroll
            for (int q = 0; q < N; ++q) dk = fma(-T->dhat[q][ax[b]], P[q * st], dk);
            dsum[k] = dk;
            tot[k] = fma(lp * nF[b][1][k], op, fma(lm * nF[b][0][k], om, tot[k]));
            if constexpr (BR2)
              vol[k] = fma(lp * nF[b][1][k], ap, fma(lm * nF[b][0][k], am, vol[k]));
          }
        }
      }
      if constexpr (!AFFINE) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          tot[k] += dsum[k];
          if constexpr (BR2) vol[k] += dsum[k];
        }
      }
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const double gt = tot[k] * jinv;
        sGt[(le * NV * DIM + v * DIM + k) * NB + node] = gt;
        if constexpr (BR2) sGv[(le * NV * DIM + v * DIM + k) * NB + node] = vol[k] * jinv;
        // artificial viscosity: the node's eps times the volume gradient (SpatialDiscrete.cpp:211-250)
        a.grad[(e * NV * DIM + v * DIM + k) * NB + node] = BR2 && a.av ? epsNode * (vol[k] * jinv) : gt;
      }
    }
  }
  __syncthreads();
  // face gradient traces
  for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
    const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
    const int f = r / NFQ, j = r - f * NFQ;
    const int axis = T->faceAxis[f], en = T->faceEnd[f];
    const double* coef = en ? T->endp : T->endm;
    const double* lift = en ? T->liftp : T->liftm;
    const int base = T->faceBase[f][j];
    const int st = strideOf<DIM, N>(axis);
    const int64_t ee = e0 + te;
    double* out = a.faceGrad + (a.faceBase + ee * NF + f) * NV * DIM * NFQ + j;
    const double* src = BR2 ? sGv : sGt;
    double nf[DIM], cl = 0.0, epsF = 1.0;
    if constexpr (BR2) {
      if (a.av) {  // eps at the face point (nodal_adjacency_value_ of the parent, SpatialDiscrete.cpp:528-631)
        double X[DIM];
#pragma unroll
        for (int c = 0; c < DIM; ++c) X[c] = c == axis ? (en ? 1.0 : -1.0) : a.avTab[axisIndex<DIM, N>(base, c)];
        epsF = vertexInterp<DIM>(a.epsV + ee * (1 << DIM), X);
      }
    }
    if constexpr (BR2) {
      // lift trace factor sum_a l_a(end)^2 / (w_a |J|_a) and the face's n|J_f|
#pragma unroll
      for (int q = 0; q < N; ++q) cl = fma(coef[q] * lift[q], sJ[te * NB + base + q * st], cl);
      if constexpr (AFFINE) {
        const double* g = a.geom + ee * GS;
#pragma unroll
        for (int k = 0; k < DIM; ++k) nf[k] = en ? g[axis * DIM + k] : -g[axis * DIM + k];
      } else {
#pragma unroll
        for (int k = 0; k < DIM; ++k)
          nf[k] = a.fmetric[(a.fmetricPoint ? (ee * NF + f) * NFQ + j : ee * NF + f) * DIM + k];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const double jump = BR2 ? sO[te * FS + (f * NV + v) * NFQ + j] - sS[te * FS + (f * NV + v) * NFQ + j] : 0.0;
#pragma unroll
      for (int k = 0; k < DIM; ++k) {
        const double* gsrc = src + (te * NV * DIM + v * DIM + k) * NB + base;
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(coef[q], gsrc[q * st], acc);
        if constexpr (BR2) acc = a.av ? epsF * acc : fma(cl * nf[k], jump, acc);
        out[(v * DIM + k) * NFQ] = acc;
      }
    }
  }
  return true;
}

template <int DIM, int N, bool AFFINE, bool BR2>
__global__ void __launch_bounds__(kMaxTileThreads) tensorGradientKernel(GradArgs a) {
  if (threadIdx.x == 0) mbarInit(tensorGradBarrier<DIM, N, AFFINE, BR2>(a.epb), 1);
  tensorGradientTile<DIM, N, AFFINE, BR2>(a, blockIdx.x, 0u, true);
}

template <int DIM, int N, bool AFFINE, bool BR2>
__global__ void __launch_bounds__(kMaxTileThreads)
    tensorGradientBatchKernel(const GradArgs* __restrict__ args, const int2* __restrict__ items, int nitems, int epb) {
  if (threadIdx.x == 0) mbarInit(tensorGradBarrier<DIM, N, AFFINE, BR2>(epb), 1);
  uint32_t parity = 0;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    const GradArgs a = args[it.x];
    if (!tensorGradientTile<DIM, N, AFFINE, BR2>(a, it.y, parity, w == int(blockIdx.x))) return;
    parity ^= 1u;
  }
}

// Interior-face Navier-Stokes flux: Riemann flux minus the central viscous flux of the two sides'
// (state, gradient) traces, times |J_f|; +/- scatter as the Euler face operation.
template <int DIM, int FLUX>
__device__ __forceinline__ void faceNSPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
  const int64_t LG = int64_t(sl) * NV * DIM * nfq + j, RG = int64_t(sr) * NV * DIM * nfq + jr;
  const Phys& ph = a.ph;
  double ul[NV], ur[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) { ul[v] = a.face[L + v * nfq]; ur[v] = a.face[R + v * nfq]; }
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
  State<DIM> l, r;
  makeState<DIM>(l, ul, ph);
  makeState<DIM>(r, ur, ph);
  double h[NV];
  convectiveFlux<DIM, FLUX>(l, r, n, ph, h);
  double fl[NV], fr[NV];
  {
    double g[NV * DIM];
#pragma unroll
    for (int c = 0; c < NV * DIM; ++c) g[c] = a.faceGrad[LG + c * nfq];
    PrimGrad<DIM> pg;
    primitiveGradient<DIM>(g, l.u, l.ir, l.E * l.ir, ph, pg);
    double u2 = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) u2 = fma(l.u[k], l.u[k], u2);
    const double T = fma(ph.incomp ? 0.0 : -0.5, u2, l.E * l.ir) * ph.inv_cv;
    viscousNormalFlux<DIM>(pg, l.u, T, n, ph, fl);
  }
  {
    double g[NV * DIM];
#pragma unroll
    for (int c = 0; c < NV * DIM; ++c) g[c] = a.faceGrad[RG + c * nfq];
    PrimGrad<DIM> pg;
    primitiveGradient<DIM>(g, r.u, r.ir, r.E * r.ir, ph, pg);
    double u2 = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) u2 = fma(r.u[k], r.u[k], u2);
    const double T = fma(ph.incomp ? 0.0 : -0.5, u2, r.E * r.ir) * ph.inv_cv;
    viscousNormalFlux<DIM>(pg, r.u, T, n, ph, fr);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = fma(-0.5, fl[v] + fr[v], h[v]) * area;
    a.faceFlux[L + v * nfq] = x;
    a.faceFlux[R + v * nfq] = negated(x);
  }
}

// Boundary-face Navier-Stokes flux (SpatialDiscrete.cpp:750-842 with modifyBoundaryVariable,
// BoundaryCondition.cpp): convective flux of the boundary state; viscous flux averaged between the
// interior side (walls: the wall state) and the boundary state, both with the interior primitive gradient
// (adiabatic walls: zero temperature gradient on the boundary side).
template <int DIM>
__device__ __forceinline__ void faceNSBoundaryPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j, LG = int64_t(sl) * NV * DIM * nfq + j;
  const Phys& ph = a.ph;
  double ul[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = a.face[L + v * nfq];
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
  State<DIM> s;
  makeState<DIM>(s, ul, ph);
  Comp<DIM> l, g, b;
  compFromState<DIM>(s, l, a.ph);
  const double* gp = a.ghost + (f * nfq + j) * (DIM + 3);
  g.r = gp[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gp[1 + k];
  g.e = gp[DIM + 1];
  g.p = gp[DIM + 2];
  boundaryState<DIM>(bc, n, l, g, ph, b);
  double h[NV];
  normalFluxComp<DIM>(b, n, h, ph);
  double gr[NV * DIM];
#pragma unroll
  for (int c = 0; c < NV * DIM; ++c) gr[c] = a.faceGrad[LG + c * nfq];
  PrimGrad<DIM> pl;
  primitiveGradient<DIM>(gr, s.u, s.ir, s.E * s.ir, ph, pl);
  const Comp<DIM>& lm = bc >= 3 ? b : l;
  double fl[NV], fb[NV];
  viscousNormalFlux<DIM>(pl, lm.u, lm.e * ph.inv_cv, n, ph, fl);
  PrimGrad<DIM> pb = pl;
  if (bc >= 4) {
#pragma unroll
    for (int k = 0; k < DIM; ++k) pb.gT[k] = 0.0;
  }
  viscousNormalFlux<DIM>(pb, b.u, b.e * ph.inv_cv, n, ph, fb);
#pragma unroll
  for (int v = 0; v < NV; ++v) a.faceFlux[L + v * nfq] = fma(-0.5, fl[v] + fb[v], h[v]) * area;
}

// Interior-face Euler flux with artificial viscosity: Riemann flux minus the central artificial viscous flux
// 1/2 (eps_L G_L + eps_R G_R).n, the gradient traces already scaled by each side's eps at the point
// (SpatialDiscrete.cpp:685-734, ViscousFlux.cpp:183-197).
template <int DIM, int FLUX>
__device__ __forceinline__ void faceAVPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  const int64_t L = int64_t(sl) * NV * nfq + j, R = int64_t(sr) * NV * nfq + jr;
  const int64_t LG = int64_t(sl) * NV * DIM * nfq + j, RG = int64_t(sr) * NV * DIM * nfq + jr;
  const Phys& ph = a.ph;
  double ul[NV], ur[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) { ul[v] = a.face[L + v * nfq]; ur[v] = a.face[R + v * nfq]; }
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
  State<DIM> l, r;
  makeState<DIM>(l, ul, ph);
  makeState<DIM>(r, ur, ph);
  double h[NV];
  convectiveFlux<DIM, FLUX>(l, r, n, ph, h);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double gl = 0.0, gr = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) {
      gl = fma(a.faceGrad[LG + (v * DIM + k) * nfq], n[k], gl);
      gr = fma(a.faceGrad[RG + (v * DIM + k) * nfq], n[k], gr);
    }
    const double x = fma(-0.5, gl + gr, h[v]) * area;
    a.faceFlux[L + v * nfq] = x;
    a.faceFlux[R + v * nfq] = negated(x);
  }
}

// Boundary-face Euler flux with artificial viscosity: normal flux of the boundary state minus the interior
// side's artificial viscous flux eps_L G_L.n (SpatialDiscrete.cpp:815-834).
template <int DIM>
__device__ __forceinline__ void faceAVBoundaryPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  const int64_t L = int64_t(sl) * NV * nfq + j, LG = int64_t(sl) * NV * DIM * nfq + j;
  const Phys& ph = a.ph;
  double ul[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = a.face[L + v * nfq];
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
  State<DIM> s;
  makeState<DIM>(s, ul, ph);
  Comp<DIM> l, g, b;
  compFromState<DIM>(s, l, ph);
  const double* gp = a.ghost + (f * nfq + j) * (DIM + 3);
  g.r = gp[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) g.u[k] = gp[1 + k];
  g.e = gp[DIM + 1];
  g.p = gp[DIM + 2];
  boundaryState<DIM>(bc, n, l, g, ph, b);
  double h[NV];
  normalFluxComp<DIM>(b, n, h, ph);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    double gl = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) gl = fma(a.faceGrad[LG + (v * DIM + k) * nfq], n[k], gl);
    a.faceFlux[L + v * nfq] = (h[v] - gl) * area;
  }
}

// ---- face-point kernels ----------------------------------------------------------------------------
template <int OP, int DIM, int FLUX>
__device__ __forceinline__ void facePointOp(const FaceArgs& a, int64_t t) {
  if constexpr (OP == kOpFace) faceInteriorPoint<DIM, FLUX>(a, t);
  else if constexpr (OP == kOpFaceBoundary) faceBoundaryPoint<DIM>(a, t);
  else if constexpr (OP == kOpExchange) exchangePoint<DIM>(a, t);
  else if constexpr (OP == kOpExchangeBoundary) exchangeBoundaryPoint<DIM>(a, t);
  else if constexpr (OP == kOpFaceNS) faceNSPoint<DIM, FLUX>(a, t);
  else if constexpr (OP == kOpFaceNSBoundary) faceNSBoundaryPoint<DIM>(a, t);
  else if constexpr (OP == kOpFaceAV) faceAVPoint<DIM, FLUX>(a, t);
  else faceAVBoundaryPoint<DIM>(a, t);
}

constexpr int kFaceThreads = 256;

template <int OP, int DIM, int FLUX>
__global__ void __launch_bounds__(kFaceThreads) facePointKernel(FaceArgs a) {
  facePointOp<OP, DIM, FLUX>(a, int64_t(blockIdx.x) * blockDim.x + threadIdx.x);
}

// Persistent batched launch over (argument set, chunk of kFaceThreads points) work items.
template <int OP, int DIM, int FLUX>
__global__ void __launch_bounds__(kFaceThreads)
    facePointBatchKernel(const FaceArgs* __restrict__ args, const int2* __restrict__ items, int nitems) {
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    facePointOp<OP, DIM, FLUX>(args[it.x], int64_t(it.y) * blockDim.x + threadIdx.x);
  }
}

}  // namespace sdg
