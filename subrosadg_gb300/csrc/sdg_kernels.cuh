// sm_103a kernels of the GB300 DG path (Euler residual, face fluxes, SSP-RK update, reductions).
//
// Data layout in HBM (one element block per element type):
//   state  U[e][v][i]            conserved v, node/basis i, element-contiguous, element stride padded to a
//                                multiple of 16 bytes so element tiles are TMA bulk-copy sources
//   face   F[slot][v][j]         one slot per (element, local face), slot = block_base + e*nface + f;
//                                holds the element's face trace between stages and its outward flux
//                                |J_f| h(U-,U+;n) after the face kernel (one writer per slot, no atomics,
//                                the scatter rule of src/Solver/SpatialDiscrete.cpp:738-744)
//   geom   affine: [e][d*d + 1]  |J| dxi_b/dx_a (row b) and 1/|J|; bilinear quads: [e][i][d*d + 1]
//
// Kernels per RK stage: faceKernel (Riemann flux on interior faces) + boundaryFaceKernel, then one
// element kernel per block that evaluates the volume term, the lift of the face fluxes, the diagonal
// mass matrix inverse and the SSP-RK combination, writes the new state and the new face traces.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "sdg_device.cuh"

namespace sdg {

constexpr uint32_t kWaitLimit = 1u << 24;

// Status word bits (host reads them after a synchronisation).
constexpr unsigned kStatusTimeout = 1u;

// ---- TMA bulk-copy helpers (cp.async.bulk + mbarrier, bounded waits) ------------------------------
__device__ __forceinline__ uint32_t smemAddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbarInit(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulkLoad(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smemAddr(dst)),
      "l"(src), "r"(bytes), "r"(smemAddr(bar))
      : "memory");
}
// Orders this thread's earlier generic-proxy accesses of shared memory before later bulk copies into it.
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// Withdraws `bytes` from the barrier's pending transaction count (bytes that no copy will deliver).
__device__ __forceinline__ void mbarCompleteTx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes) : "memory");
}
// Bounded wait on phase `parity` (at most `limit` try_wait rounds); returns false (and the caller flags a
// timeout) if it never completes.
__device__ __forceinline__ bool mbarWait(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  for (uint32_t it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ---- parameter blocks -----------------------------------------------------------------------------
// Operator tables of a tensor block, copied into shared memory by every CTA (size a multiple of 8).
struct TensorTables {
  double dhat[6][6];
  double endm[6], endp[6], liftm[6], liftp[6];
  double w[6];
  double b1[6][6];
  int faceAxis[6], faceEnd[6];   // normal axis and end (0: -1, 1: +1) of each local face
  int axisFace[3][2];            // local face of (axis, end)
  int faceBase[6][36];           // first node of the line through face point j of face f
  unsigned char nodeFacePoint[3][2][216];  // face point of (axis, end) on the line through node i
};
static_assert(sizeof(TensorTables) % 8 == 0, "TensorTables must be a whole number of doubles");

struct StageArgs {
  const double* uin;      // stage input state
  const double* ubase;    // RK base state (U at the start of the step)
  double* uout;           // new state
  double* face;           // face buffer (this block's slots start at face + faceBase)
  const double* geom;
  const double* tables;   // TensorTables or dense tables (device)
  double* rate;           // optional du/dt output at the volume points ([e][q][v]), or null
  double* relerr;         // optional per-CTA partial sums [cta][v], or null
  unsigned* status;
  int64_t ne;
  int64_t faceBase;       // first slot of this block
  double c0, c1, c2dt;    // U = c1 U + c0 U0 + c2 dt M^-1 R
  int doUpdate;           // 0: no state update (rate/trace only)
  int doTrace;            // write new face traces
  int doVolume;           // evaluate the residual (0: trace-only pass)
  const double* fluxSrc;  // face-flux slots to lift (null: the face buffer itself, the Euler layout)
  const double* grad;     // Navier-Stokes: total gradient at the nodes [e][nv*d][NB]; artificial viscosity:
                          // tensor blocks eps times the volume gradient at the nodes, dense blocks the modal
                          // volume-gradient coefficients
  int epb;                // elements per CTA tile (tile t covers elements [t*epb, t*epb + epb))
  int av;                 // artificial viscosity (the viscous variant with the flux eps grad U)
  const double* epsV;     // artificial viscosity at the element vertices [e][nvert]
  const double* avTab;    // artificial-viscosity tables of the block (avTableLayout)
  // Check of the bounded wait (sdg_set_wait_check): extra bytes declared to the tile's mbarrier beyond what
  // its copies carry, so that the wait can end only by its limit; and that limit (0: kWaitLimit rounds).
  unsigned txExtra;
  unsigned waitLimit;
  int diagMetric;         // affine block with diagonal metric terms only (structured axis-aligned boxes)
  int pad;
  double* pointsOut;      // tensor blocks, updating stages: also write the new state in point layout ([e][q][v])
                          // here (a pinned host buffer the device maps), or null
};

// Artificial-viscosity tables of a block (doubles):
//   tensor: x[N] (Gauss nodes on [-1,1]) | w[N] | phi1[N][N] (lob_m(x_i)) | phi1inv[N][N]
//   dense : phi[NQ][NB] | high[NB] (1 for the modes of degree P) | w[NQ] | nodal[NQ][NVERT] | nodalf[NFP][NVERT]
// nodal / nodalf: the first-order nodal (vertex) basis at the volume and face points.
inline __host__ __device__ int avDenseNodalOffset(int nb, int nq) { return nq * nb + nb + nq; }
inline __host__ __device__ int avDenseNodalFaceOffset(int nb, int nq, int nvert) {
  return avDenseNodalOffset(nb, nq) + nq * nvert;
}

// Per-step artificial viscosity (SpatialDiscrete.cpp:37-124): kind 0 zeroes the node field, 1 / 2 run the
// sensor of a tensor / dense block (max into the nodes), 3 gathers the vertex values of a block.
struct AvArgs {
  const double* u;        // block state
  const double* geom;     // block geometry (the stage kernel's layout)
  const int* vert;        // [e][nvert] mesh node of each vertex
  const double* inner;    // [e] inner radius
  const double* tab;      // avTableLayout
  double* nodeAV;         // [nodes]
  double* epsV;           // [e][nvert]
  int64_t ne, nodes;
  int kind, dim, n, nb, nq, nvert, ustride, affine, p, pad;
  double s0, kappa, factor;
};

// Points per face: 1 (the point faces of a line), N (quadrangle edges), N^2 (hexahedron faces).  Triangular
// faces (tetrahedra) carry n1d = -(points per face) and pair their points through a permutation table.
template <int DIM>
__host__ __device__ __forceinline__ constexpr int nfqOf(int n1d) {
  return DIM == 1 ? 1 : (DIM == 2 ? n1d : (n1d < 0 ? -n1d : n1d * n1d));
}

template <int DIM, int N>
struct TensorShape {
  static constexpr int NV = DIM + 2;
  static constexpr int NB = DIM == 1 ? N : (DIM == 2 ? N * N : N * N * N);
  static constexpr int NF = 2 * DIM;
  static constexpr int NFQ = nfqOf<DIM>(N);
  static constexpr int USTRIDE = (NV * NB + 1) & ~1;
  static constexpr int FSTRIDE = NF * NV * NFQ;
  static constexpr int EPB_RAW = 256 / NB > 0 ? 256 / NB : 1;
  // elements per CTA, bounded so the CTA's shared memory stays under ~96 KB (two CTAs per SM at least)
  static constexpr int SMEM_PER_ELEM = 8 * (USTRIDE + DIM * NV * NB + FSTRIDE);
  static constexpr int EPB_SMEM = (96 * 1024) / SMEM_PER_ELEM > 0 ? (96 * 1024) / SMEM_PER_ELEM : 1;
  static constexpr int EPB = EPB_RAW < EPB_SMEM ? EPB_RAW : EPB_SMEM;
  static constexpr int THREADS = ((EPB * NB + 31) / 32) * 32;
  static constexpr size_t SMEM = size_t(EPB) * SMEM_PER_ELEM + sizeof(TensorTables) + 16 + 8 * NV * (THREADS / 32);
  // any tile size: one thread per node, rounded up to whole warps
  static constexpr int threadsFor(int epb) { return ((epb * NB + 31) / 32) * 32; }
  static constexpr size_t smemFor(int epb) {
    return size_t(epb) * SMEM_PER_ELEM + sizeof(TensorTables) + 16 + 8 * NV * size_t(threadsFor(epb) / 32);
  }
};

constexpr int kMaxTileThreads = 512;

// Index of node i along axis a.
template <int DIM, int N>
__device__ __forceinline__ int axisIndex(int i, int a) {
  if constexpr (DIM == 1) return i;
  else if constexpr (DIM == 2) return a == 0 ? i / N : i % N;
  else return a == 0 ? i / (N * N) : (a == 1 ? (i / N) % N : i % N);
}

template <int DIM, int N>
__device__ __forceinline__ int strideOf(int a) {
  if constexpr (DIM == 1) return 1;
  else if constexpr (DIM == 2) return a == 0 ? N : 1;
  else return a == 0 ? N * N : (a == 1 ? N : 1);
}

// Tensor-block stage tile: one thread per node, a.epb elements per CTA.  Shared memory (dynamic):
// sU [epb][USTRIDE] | sF [epb][FSTRIDE] | sG [epb][DIM][NV][NB] | TensorTables | mbarrier | [warps][NV] (spare).
template <int DIM, int N>
__device__ __forceinline__ uint64_t* tensorStageBarrier(int epb) {
  using S = TensorShape<DIM, N>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sG = reinterpret_cast<double*>(smem_raw) + epb * (S::USTRIDE + S::FSTRIDE);
  return reinterpret_cast<uint64_t*>(reinterpret_cast<TensorTables*>(sG + epb * DIM * S::NV * S::NB) + 1);
}

// One tile of a stage: the CTA's mbarrier is initialised, `parity` is the phase this tile's copies complete;
// `loadTables` copies the operator tables (identical for every tile of a (type, order) variant).  Returns
// false after a timed-out copy (status flagged, every thread returns together).
template <int DIM, int N, bool AFFINE, int VISC>
__device__ __forceinline__ bool tensorStageTile(const StageArgs& a, const Phys& ph, int64_t tile, uint32_t parity,
                                                bool loadTables) {
  using S = TensorShape<DIM, N>;
  constexpr int NV = S::NV, NB = S::NB, NF = S::NF, NFQ = S::NFQ;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int epb = a.epb;
  double* sU = reinterpret_cast<double*>(smem_raw);                 // [epb][USTRIDE]
  double* sF = sU + epb * S::USTRIDE;                               // [epb][FSTRIDE]
  double* sG = sF + epb * S::FSTRIDE;                               // [epb][DIM][NV][NB]
  TensorTables* T = reinterpret_cast<TensorTables*>(sG + epb * DIM * NV * NB);
  uint64_t* bar = reinterpret_cast<uint64_t*>(T + 1);

  const int tid = threadIdx.x;
  const int64_t e0 = tile * epb;
  const int ecount = int(a.ne - e0 < epb ? a.ne - e0 : epb);
  const int le = tid / NB, node = tid - le * NB;
  const bool active = le < ecount;
  const int64_t e = e0 + le;

  __syncthreads();  // the previous tile's readers of sU/sF are done
  // 1. stage the element tile (state + face slots) into shared memory with TMA bulk copies
  if (tid == 0) {
    fenceProxyAsync();
    const uint32_t ub = uint32_t(ecount) * S::USTRIDE * 8, fb = uint32_t(ecount) * S::FSTRIDE * 8;
    mbarExpectTx(bar, (a.doVolume ? ub + fb : ub) + a.txExtra);
    bulkLoad(sU, a.uin + e0 * S::USTRIDE, ub, bar);
    if (a.doVolume) bulkLoad(sF, (a.fluxSrc ? a.fluxSrc : a.face) + (a.faceBase + e0 * NF) * NV * NFQ, fb, bar);
  }
  if (loadTables) {
    const double* src = a.tables;
    double* dst = reinterpret_cast<double*>(T);
    for (int k = tid; k < int(sizeof(TensorTables) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const bool arrived = mbarWait(bar, parity, a.waitLimit ? a.waitLimit : kWaitLimit);
  if (__syncthreads_or(!arrived)) {  // uniform decision: every thread leaves together
    if (tid == 0) {
      atomicOr(a.status, kStatusTimeout);
      if (a.txExtra) mbarCompleteTx(bar, a.txExtra);  // the phase now completes once the real copies land
      mbarWait(bar, parity);  // bounded: let copies still in flight land before the CTA exits
    }
    return false;
  }

  double du[NV];
  double unew[NV];
  if (a.doVolume) {
    // 2. contravariant fluxes at the node
    double jinv;
    double ja[DIM][DIM];
    if (active) {
      const double* g = AFFINE ? a.geom + e * (DIM * DIM + 1) : a.geom + (e * NB + node) * (DIM * DIM + 1);
#pragma unroll
      for (int b = 0; b < DIM; ++b)
#pragma unroll
        for (int c = 0; c < DIM; ++c) ja[b][c] = g[b * DIM + c];
      jinv = g[DIM * DIM];
      double U[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) U[v] = sU[le * S::USTRIDE + v * NB + node];
      State<DIM> s;
      makeState<DIM>(s, U, ph);
      const double ep = energyFluxFactor(s, ph);
      double tau[DIM][DIM], q[DIM];
      double gv[VISC ? NV * DIM : 1];
      if constexpr (VISC != 0) {
        // Navier-Stokes: viscous flux from the total gradient at the node (ViscousFlux.cpp:58-103);
        // artificial viscosity: the gradient kernel stored eps times the volume gradient, the flux itself
        // (ViscousFlux.cpp:105-113)
#pragma unroll
        for (int c = 0; c < NV * DIM; ++c) gv[c] = a.grad[(e * NV * DIM + c) * NB + node];
      }
      if constexpr (VISC == 1) {
        PrimGrad<DIM> pg;
        primitiveGradient<DIM>(gv, s.u, s.ir, s.E * s.ir, ph, pg);
        double u2 = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; ++k) u2 = fma(s.u[k], s.u[k], u2);
        viscousTensor<DIM>(pg, s.u, fma(ph.incomp ? 0.0 : -0.5, u2, s.E * s.ir) * ph.inv_cv, ph,
                           tau, q);
      }
      if (AFFINE && a.diagMetric) {
        // axis-aligned element: ja[b][c] = 0 for c != b.  The same products as the general form below
        // without its multiplications by zero (every skipped term is an exact +-0): equal values, at most
        // the sign of an exact zero differs.
#pragma unroll
        for (int b = 0; b < DIM; ++b) {
          const double jb = ja[b][b];
          const double vb = s.u[b] * jb;
          double* G = sG + ((le * DIM + b) * NV) * NB + node;
          G[0] = s.r * vb;
#pragma unroll
          for (int k = 0; k < DIM; ++k) {
            double x = k == b ? fma(s.m[k], vb, jb * s.p) : s.m[k] * vb;
            if constexpr (VISC == 1) x = fma(-jb, tau[b][k], x);
            G[(1 + k) * NB] = x;
          }
          double xe = ep * vb;
          if constexpr (VISC == 1) xe -= q[b] * jb;
          G[(NV - 1) * NB] = xe;
          if constexpr (VISC == 2) {
#pragma unroll
            for (int v = 0; v < NV; ++v) G[v * NB] = fma(-jb, gv[v * DIM + b], G[v * NB]);
          }
        }
      } else {
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const double vb = dotn<DIM>(s.u, ja[b]);
        double* G = sG + ((le * DIM + b) * NV) * NB + node;
        G[0] = s.r * vb;
#pragma unroll
        for (int k = 0; k < DIM; ++k) {
          double x = fma(s.m[k], vb, ja[b][k] * s.p);
          if constexpr (VISC == 1) {
#pragma unroll
            for (int c = 0; c < DIM; ++c) x = fma(-ja[b][c], tau[c][k], x);
          }
          G[(1 + k) * NB] = x;
        }
        double xe = ep * vb;
        if constexpr (VISC == 1) xe -= dotn<DIM>(q, ja[b]);
        G[(NV - 1) * NB] = xe;
        if constexpr (VISC == 2) {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            double x = G[v * NB];
#pragma unroll
            for (int c = 0; c < DIM; ++c) x = fma(-ja[b][c], gv[v * DIM + c], x);
            G[v * NB] = x;
          }
        }
      }
      }
    }
    __syncthreads();
    // 3. weak derivative along each axis + lift of the face fluxes (mass-scaled), per node
    if (active) {
      int ax[DIM];
#pragma unroll
      for (int b = 0; b < DIM; ++b) ax[b] = axisIndex<DIM, N>(node, b);
#pragma unroll
      for (int v = 0; v < NV; ++v) du[v] = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const int base = node - ax[b] * strideOf<DIM, N>(b);
        double dcoef[N];
#pragma unroll
        for (int q = 0; q < N; ++q) dcoef[q] = T->dhat[q][ax[b]];
        const double lm = T->liftm[ax[b]], lp = T->liftp[ax[b]];
        const int fm = T->axisFace[b][0], fp = T->axisFace[b][1];
        const int jm = T->nodeFacePoint[b][0][node], jp = T->nodeFacePoint[b][1][node];
        const double* G = sG + ((le * DIM + b) * NV) * NB + base;
        const double* Fm = sF + le * S::FSTRIDE + fm * NV * NFQ + jm;
        const double* Fp = sF + le * S::FSTRIDE + fp * NV * NFQ + jp;
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          double acc = du[v];
#pragma unroll
          for (int q = 0; q < N; ++q) acc = fma(dcoef[q], G[v * NB + q * strideOf<DIM, N>(b)], acc);
          acc = fma(-lm, Fm[v * NFQ], acc);
          acc = fma(-lp, Fp[v * NFQ], acc);
          du[v] = acc;
        }
      }
      // Boussinesq buoyancy on the last momentum component (SourceTerm.cpp:29-58): the nodal source S_i
      // enters as S_i |J|_i (it is divided by w_i |J|_i with the rest of the residual)
      if (ph.source) {
        double U[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v) U[v] = sU[le * S::USTRIDE + v * NB + node];
        State<DIM> s;
        makeState<DIM>(s, U, ph);
        du[DIM] = fma(s.r * ph.beta * (temperatureOf(s, ph) - ph.tref), 1.0 / jinv, du[DIM]);
      }
      // 4. RK combination (M^-1 is diagonal: 1/(w_i |J|_i); the weights cancelled into dhat/lift)
      const double sc = a.c2dt * jinv;
      const int64_t gi = e * S::USTRIDE + node;
      if (a.rate) {
        // reference point order equals the node order for tensor blocks
#pragma unroll
        for (int v = 0; v < NV; ++v) a.rate[(e * NB + node) * NV + v] = du[v] * jinv;
      }
      if (a.doUpdate) {
        if (a.uin == a.ubase && a.c1 == 0.0 && a.c0 == 1.0) {
          // first stage of a step (every RK table starts with {1, 0, 1}): U = U^n + dt M^-1 R, and U^n is
          // the staged tile itself, so the base state is not read again
#pragma unroll
          for (int v = 0; v < NV; ++v) unew[v] = fma(sc, du[v], sU[le * S::USTRIDE + v * NB + node]);
        } else {
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            const double u0 = a.ubase[gi + v * NB];
            const double u1 = sU[le * S::USTRIDE + v * NB + node];
            unew[v] = fma(sc, du[v], fma(a.c1, u1, a.c0 * u0));
          }
        }
      }
    }
    __syncthreads();
    // relative error (TimeIntegration.cpp:279-324): the nodal weak residual is R_i = M_ii du_i = w_i * bracket_i
    // (jinv was not applied to du); rel = (B1 x B1 [x B1]) R with B1(a,b) = sum_k lob_k(x_a) lob_k(x_b), the
    // tensor form of Phi Phi^T for the modal basis; per element the mean over points of |rel| is summed.
    if (a.relerr) {
      if (active) {
        double wi = 1.0;
#pragma unroll
        for (int b = 0; b < DIM; ++b) wi *= T->w[axisIndex<DIM, N>(node, b)];
        double* R0 = sG + le * DIM * NV * NB;
#pragma unroll
        for (int v = 0; v < NV; ++v) R0[v * NB + node] = wi * du[v];
      }
      __syncthreads();
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        const double* in = sG + le * DIM * NV * NB + (b & 1) * NV * NB;
        double* out = sG + le * DIM * NV * NB + ((b + 1) & 1) * NV * NB;
        double r[NV];
        if (active) {
          const int ib = axisIndex<DIM, N>(node, b);
          const int st = strideOf<DIM, N>(b);
          const int base = node - ib * st;
#pragma unroll
          for (int v = 0; v < NV; ++v) {
            double acc = 0.0;
#pragma unroll
            for (int q = 0; q < N; ++q) acc = fma(T->b1[ib][q], in[v * NB + base + q * st], acc);
            r[v] = acc;
          }
        }
        __syncthreads();
        if (active) {
#pragma unroll
          for (int v = 0; v < NV; ++v) out[v * NB + node] = r[v];
        }
        __syncthreads();
      }
      // deterministic reduction: warp v sums variable v's |rel| over the tile's nodes straight from shared
      // memory (a strided pass per lane, then one shuffle tree), so each variable costs one warp's work
      // instead of a shuffle tree in every warp
      {
        const int warp = tid >> 5, lane = tid & 31, nwarp = (blockDim.x + 31) >> 5;
        const double* fin = sG + (DIM & 1) * NV * NB;
        for (int v = warp; v < NV; v += nwarp) {
          double x = 0.0;
          for (int k = lane; k < ecount * NB; k += 32) {
            const int te = k / NB;
            x += fabs(fin[te * DIM * NV * NB + v * NB + (k - te * NB)]);
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
          if (lane == 0) a.relerr[tile * NV + v] = x / double(NB);
        }
      }
    }
    if (a.doUpdate && active) {
      const int64_t gi = e * S::USTRIDE + node;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        a.uout[gi + v * NB] = unew[v];
        sU[le * S::USTRIDE + v * NB + node] = unew[v];
      }
    }
    __syncthreads();
    if (a.doUpdate && a.pointsOut) {
      // the tile's new state as one contiguous run of the point layout (nodes are the volume points):
      // consecutive threads on consecutive addresses, so host-memory writes over the CPU-GPU link go out whole
      double* dst = a.pointsOut + e0 * (NB * NV);
      for (int i = tid; i < ecount * (NB * NV); i += blockDim.x) {
        const int te = i / (NB * NV), r = i - te * (NB * NV), q = r / NV, v = r - q * NV;
        dst[i] = sU[te * S::USTRIDE + v * NB + q];
      }
    }
  }
  // 5. face traces of the (new) state: 1D end-point interpolation along each face's normal axis
  if (a.doTrace) {
    for (int idx = tid; idx < ecount * NF * NFQ; idx += blockDim.x) {
      const int te = idx / (NF * NFQ), r = idx - te * (NF * NFQ);
      const int f = r / NFQ, j = r - f * NFQ;
      const int axis = T->faceAxis[f];
      const double* coef = T->faceEnd[f] ? T->endp : T->endm;
      const int base = T->faceBase[f][j];
      const int st = strideOf<DIM, N>(axis);
      const double* u = sU + te * S::USTRIDE + base;
      double* out = a.face + (a.faceBase + (e0 + te) * NF + f) * NV * NFQ + j;
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        double acc = 0.0;
#pragma unroll
        for (int q = 0; q < N; ++q) acc = fma(coef[q], u[v * NB + q * st], acc);
        out[v * NFQ] = acc;
      }
    }
  }
  return true;
}

// One CTA per tile.
template <int DIM, int N, bool AFFINE, int VISC>
__global__ void __launch_bounds__(kMaxTileThreads) tensorStageKernel(StageArgs a, Phys ph) {
  if (threadIdx.x == 0) mbarInit(tensorStageBarrier<DIM, N>(a.epb), 1);
  tensorStageTile<DIM, N, AFFINE, VISC>(a, ph, blockIdx.x, 0u, true);
}

// Persistent batched launch: CTA c runs work items c, c + gridDim.x, ... of a list of (argument set, tile)
// pairs that spans many independent instances of one (type, order) variant.  The barrier is initialised
// once and its phase alternates per tile; the tables are loaded once per CTA.
template <int DIM, int N, bool AFFINE, int VISC>
__global__ void __launch_bounds__(kMaxTileThreads)
    tensorStageBatchKernel(const StageArgs* __restrict__ args, const Phys* __restrict__ phys,
                           const int2* __restrict__ items, int nitems, int epb) {
  if (threadIdx.x == 0) mbarInit(tensorStageBarrier<DIM, N>(epb), 1);
  uint32_t parity = 0;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const int2 it = items[w];
    const StageArgs a = args[it.x];
    const Phys ph = phys[it.x];
    if (!tensorStageTile<DIM, N, AFFINE, VISC>(a, ph, it.y, parity, w == int(blockIdx.x))) return;
    parity ^= 1u;
  }
}

// ---- face-point operations -----------------------------------------------------------------------
// One thread per face point; the same argument block serves the one-instance kernels and the batched
// persistent kernels.  Slot layout: see the file header.
struct FaceArgs {
  double* face;              // traces (the Euler flux operations overwrite them with |J_f| h)
  double* other;             // Navier-Stokes: neighbour traces
  const double* faceGrad;    // Navier-Stokes: gradient traces [slot][v*d+k][j]
  double* faceFlux;          // Navier-Stokes: face fluxes
  const int* conn;           // interior: (slot L, slot R, rotation); boundary: (slot, condition, 0)
  const int* perm;           // triangular faces: right point of left point j at rotation r, [3][nfq]
  const double* fgeo;        // per face (n, |J_f|)
  const double* ghost;       // boundary: [face][j][rho, u, e, p]
  int64_t nface;
  int n1d;
  int fgeoPoint;             // 1: fgeo per face point [face][j][n, |J_f|] (curved meshes); 0: per face
  Phys ph;
};

// (n, |J_f|) of face point j of face f: per face, or per point on curved meshes.
__device__ __forceinline__ const double* faceGeometry(const double* fgeo, int fgeoPoint, int64_t f, int j, int nfq) {
  return fgeo + (fgeoPoint ? (f * nfq + j) * 4 : f * 4);
}

enum FaceOp { kOpFace = 0, kOpFaceBoundary = 1, kOpExchange = 2, kOpExchangeBoundary = 3, kOpFaceNS = 4,
              kOpFaceNSBoundary = 5, kOpFaceAV = 6, kOpFaceAVBoundary = 7 };
constexpr int kFaceOps = 8;

// Point of the right face that coincides with point j of the left face (rotation of the right face's
// vertex list; SimulationControl.cpp:381-523 permutations).
template <int DIM>
__host__ __device__ __forceinline__ int rightPoint(int j, int rot, int n1d) {
  if constexpr (DIM == 1) {
    return 0;
  } else if constexpr (DIM == 2) {
    return n1d - 1 - j;
  } else {
    const int i = j / n1d, k = j - i * n1d;
    int ii, kk;
    switch (rot) {
      case 0: ii = k; kk = i; break;
      case 1: ii = n1d - 1 - i; kk = k; break;
      case 2: ii = n1d - 1 - k; kk = n1d - 1 - i; break;
      default: ii = i; kk = n1d - 1 - k; break;
    }
    return ii * n1d + kk;
  }
}

// Right point of left point j on an interior face: the tensor rotation, or the permutation table of
// triangular faces (n1d < 0).
template <int DIM, class Args>
__device__ __forceinline__ int pairedPoint(const Args& a, int j, int rot, int nfq) {
  return (DIM == 3 && a.n1d < 0) ? a.perm[rot * nfq + j] : rightPoint<DIM>(j, rot, a.n1d);
}

// Interior-face Riemann flux.  Left slot gets +|J_f| h, right slot gets -|J_f| h at the permuted point
// (SpatialDiscrete.cpp:633-748).
template <int DIM, int FLUX>
__device__ __forceinline__ void faceInteriorPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], sr = a.conn[f * 3 + 1], rot = a.conn[f * 3 + 2];
  const int jr = pairedPoint<DIM>(a, j, rot, nfq);
  double* L = a.face + int64_t(sl) * NV * nfq + j;
  double* R = a.face + int64_t(sr) * NV * nfq + jr;
  double ul[NV], ur[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) { ul[v] = L[v * nfq]; ur[v] = R[v * nfq]; }
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
  State<DIM> l, r;
  makeState<DIM>(l, ul, a.ph);
  makeState<DIM>(r, ur, a.ph);
  double h[NV];
  convectiveFlux<DIM, FLUX>(l, r, n, a.ph, h);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const double x = h[v] * area;
    L[v * nfq] = x;
    R[v * nfq] = negated(x);
  }
}

// Boundary-face flux: ghost state from the boundary condition, normal flux of the boundary state
// (SpatialDiscrete.cpp:750-842).
template <int DIM>
__device__ __forceinline__ void faceBoundaryPoint(const FaceArgs& a, int64_t t) {
  constexpr int NV = DIM + 2;
  const int n1d = a.n1d;
  const int nfq = nfqOf<DIM>(n1d);
  const int64_t f = t / nfq;
  if (f >= a.nface) return;
  const int j = int(t - f * nfq);
  const int sl = a.conn[f * 3 + 0], bc = a.conn[f * 3 + 1];
  double* L = a.face + int64_t(sl) * NV * nfq + j;
  double ul[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v) ul[v] = L[v * nfq];
  double n[DIM];
  const double* fg = faceGeometry(a.fgeo, a.fgeoPoint, f, j, nfq);
#pragma unroll
  for (int k = 0; k < DIM; ++k) n[k] = fg[k];
  const double area = fg[3];
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
  double h[NV];
  normalFluxComp<DIM>(b, n, h, a.ph);
#pragma unroll
  for (int v = 0; v < NV; ++v) L[v * nfq] = h[v] * area;
}

// Deterministic final reduction of per-tile relative-error partials: out[v] = sum / elements.
struct RelArgs {
  const double* part;        // [slot][nv]
  int64_t offset[2], count[2];  // used slot ranges (one per element block)
  double* out;
  double inv_elements;
  int nranges, nv;
};

}  // namespace sdg
