// C ABI of the GB300 DG path (include/sdg_gpu.h): problem setup, device buffers, launches.
//
// sdg_create replaces Mesh<SC>::readMeshElement + Solver<SC> construction
// (src/Mesh/ReadControl.cpp:293-335, src/Solver/InitialCondition.cpp:151-186); sdg_step replaces
// Solver<SC>::stepSolver (src/Solver/TimeIntegration.cpp:326-350).  Every failure is returned as an
// SDG_ERR_* code with text in sdg_last_error; nothing falls back to the CPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <map>
#include <mutex>
#include <set>

#include "sdg_geometry.hpp"
#include "sdg_internal.hpp"

namespace sdg {

// Independent-chain FP64 FMA kernel (bounded loop, no waits): measures the FP64 pipe throughput.
__global__ void fp64ProbeKernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 8; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core (DMMA) issue probe: every warp runs CHAINS independent accumulator chains of
// mma.sync .f64 of one shape (bounded loop, no waits, registers only).  SHAPE 0: m8n8k4 (sm_80 form),
// 1: m16n8k4, 2: m16n8k8, 3: m16n8k16 (the sm_90+ forms).  The operands are tiny so nothing overflows.
template <int SHAPE>
__global__ void dmmaProbeKernel(double* out, int iters) {
  constexpr int CHAINS = 4;
  const double a = 1e-9 * double(threadIdx.x & 31), b = 1e-9;
  double acc[CHAINS][4];
#pragma unroll
  for (int c = 0; c < CHAINS; ++c)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[c][r] = 0.0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) {
      if constexpr (SHAPE == 0) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(acc[c][0]), "+d"(acc[c][1]) : "d"(a), "d"(b));
      } else if constexpr (SHAPE == 1) {
        asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                     : "+d"(acc[c][0]), "+d"(acc[c][1]), "+d"(acc[c][2]), "+d"(acc[c][3]) : "d"(a), "d"(a), "d"(b));
      } else if constexpr (SHAPE == 2) {
        asm volatile("mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};"
                     : "+d"(acc[c][0]), "+d"(acc[c][1]), "+d"(acc[c][2]), "+d"(acc[c][3])
                     : "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b));
      } else {
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                     "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
                     : "+d"(acc[c][0]), "+d"(acc[c][1]), "+d"(acc[c][2]), "+d"(acc[c][3])
                     : "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b), "d"(b), "d"(b));
      }
    }
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < CHAINS; ++c)
#pragma unroll
    for (int r = 0; r < 4; ++r) s += acc[c][r];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

void facePointInParent(int type, int f, const double* fx, double* X) {
  const int nfv = typeFaceVertices(type);
  const int* fl = faceVertexList(type);
  double sh[4];
  if (nfv == 1) sh[0] = 1.0;
  else if (nfv == 2) { sh[0] = 0.5 * (1 - fx[0]); sh[1] = 0.5 * (1 + fx[0]); }
  else if (nfv == 3) { sh[0] = 1 - fx[0] - fx[1]; sh[1] = fx[0]; sh[2] = fx[1]; }
  else {
    const double x = fx[0], y = fx[1];
    sh[0] = 0.25 * (1 - x) * (1 - y); sh[1] = 0.25 * (1 + x) * (1 - y);
    sh[2] = 0.25 * (1 + x) * (1 + y); sh[3] = 0.25 * (1 - x) * (1 + y);
  }
  X[0] = X[1] = X[2] = 0.0;
  for (int k = 0; k < nfv; ++k) {
    double V[3]; referenceVertex(type, fl[f * nfv + k], V);
    for (int d = 0; d < 3; ++d) X[d] += sh[k] * V[d];
  }
}

// Outward n|J_f| (unnormalised) at face point fx of local face f, from the parent's Jacobian J there: the
// face's tangents are J times the derivatives of its P1 map into the parent's reference element (the map of
// facePointInParent); edges: n|J_f| = (t_y, -t_x); quadrangle and triangle faces: n|J_f| = t_xi x t_eta
// (Geometry.cpp:115-147).  For a straight-sided parent this is the face's own P1 map differentiated.
void faceNormalScaled(int type, int f, const double* fx, const double J[3][3], double* nJ) {
  const int nfv = typeFaceVertices(type);
  const int* fl = faceVertexList(type);
  double ds[4] = {0, 0, 0, 0}, dt[4] = {0, 0, 0, 0};
  if (nfv == 2) { ds[0] = -0.5; ds[1] = 0.5; }
  else if (nfv == 3) { ds[0] = -1.0; ds[1] = 1.0; dt[0] = -1.0; dt[2] = 1.0; }
  else if (nfv == 4) {
    const double x = fx[0], y = fx[1];
    ds[0] = -0.25 * (1 - y); ds[1] = 0.25 * (1 - y); ds[2] = 0.25 * (1 + y); ds[3] = -0.25 * (1 + y);
    dt[0] = -0.25 * (1 - x); dt[1] = -0.25 * (1 + x); dt[2] = 0.25 * (1 + x); dt[3] = 0.25 * (1 - x);
  }
  double dXs[3] = {0, 0, 0}, dXt[3] = {0, 0, 0};
  for (int k = 0; k < nfv; ++k) {
    double V[3]; referenceVertex(type, fl[f * nfv + k], V);
    for (int d = 0; d < 3; ++d) { dXs[d] += ds[k] * V[d]; dXt[d] += dt[k] * V[d]; }
  }
  double t1[3] = {0, 0, 0}, t2[3] = {0, 0, 0};
  for (int l = 0; l < 3; ++l)
    for (int k = 0; k < 3; ++k) { t1[l] += J[l][k] * dXs[k]; t2[l] += J[l][k] * dXt[k]; }
  if (nfv == 2) { nJ[0] = t1[1]; nJ[1] = -t1[0]; nJ[2] = 0.0; return; }
  nJ[0] = t1[1] * t2[2] - t1[2] * t2[1];
  nJ[1] = t1[2] * t2[0] - t1[0] * t2[2];
  nJ[2] = t1[0] * t2[1] - t1[1] * t2[0];
}

// Face-point pairing of triangular faces (the Triangle cases of SimulationControl.cpp:405-434, derived from
// the geometry): the right face lists the shared vertices in the opposite orientation with the left face's
// first vertex at position r, so left point (xi, eta) is right point r=0: (eta, xi), r=1: (1-xi-eta, eta),
// r=2: (xi, 1-xi-eta).  Returns [3][nfq].
std::vector<int> triangleFacePermutation(int type, int p) {
  const PointRule fr = faceRule(type, p);
  std::vector<int> perm(size_t(3) * fr.n, -1);
  for (int r = 0; r < 3; ++r)
    for (int j = 0; j < fr.n; ++j) {
      const double x = fr.x[j * 3], y = fr.x[j * 3 + 1];
      const double X = r == 0 ? y : (r == 1 ? 1 - x - y : x), Y = r == 0 ? x : (r == 1 ? y : 1 - x - y);
      for (int k = 0; k < fr.n; ++k)
        if (std::fabs(fr.x[k * 3] - X) < 1e-12 && std::fabs(fr.x[k * 3 + 1] - Y) < 1e-12) perm[size_t(r) * fr.n + j] = k;
      if (perm[size_t(r) * fr.n + j] < 0) throw Failure(SDG_ERR_INVALID_ARGUMENT, "face rule is not symmetric");
    }
  return perm;
}

// ---- point-layout conversions ----------------------------------------------------------------------
// state[e][v][b] (padded stride) <- points[e][q][v]; proj = null for tensor blocks (nodes are points),
// else the least-squares projection [nb][nq] followed by its row sums [nb].  The projection is applied to
// u - u_0 (u_0 = the element's first point value) and u_0 added back through the row sums: for nearly uniform
// fields (the weakly compressible density, whose c0^2 amplification reaches the pressure) the rounding then
// scales with the variation of u, not with u.
__global__ void pointToStateKernel(const double* __restrict__ pts, double* __restrict__ st,
                                   const double* __restrict__ proj, int64_t ne, int nb, int nq, int nv, int ustride) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ne * nb) return;
  const int64_t e = t / nb;
  const int b = int(t - e * nb);
  for (int v = 0; v < nv; ++v) {
    double s;
    if (!proj) s = pts[(e * nq + b) * nv + v];
    else {
      const double u0 = pts[(e * nq) * nv + v];
      s = 0.0;
      for (int q = 0; q < nq; ++q) s = fma(proj[b * nq + q], pts[(e * nq + q) * nv + v] - u0, s);
      s = fma(proj[nb * nq + b], u0, s);
    }
    st[e * ustride + v * nb + b] = s;
  }
}

__global__ void stateToPointKernel(const double* __restrict__ st, double* __restrict__ pts,
                                   const double* __restrict__ phi, int64_t ne, int nb, int nq, int nv, int ustride) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ne * nq) return;
  const int64_t e = t / nq;
  const int q = int(t - e * nq);
  for (int v = 0; v < nv; ++v) {
    double s;
    if (!phi) s = st[e * ustride + v * nb + q];
    else { s = 0.0; for (int b = 0; b < nb; ++b) s = fma(phi[q * nb + b], st[e * ustride + v * nb + b], s); }
    pts[(e * nq + q) * nv + v] = s;
  }
}

// Point layout of a buffer that may be host memory the GPU reaches over the CPU-GPU link: per CTA a run of
// whole elements, the point-layout side read or written as one contiguous stretch (consecutive threads,
// consecutive addresses), the state-layout side through shared memory.  tile: [elements][nq][nv].
// pointsToTensorStateKernel: tensor blocks (points are the nodes) from points to state;
// stateToPointsTiledKernel: any block from state to points (phi null: tensor, else the dense Phi).
__global__ void pointsToTensorStateKernel(const double* __restrict__ pts, double* __restrict__ st, int64_t ne, int nb,
                                          int nv, int ustride, int epc) {
  extern __shared__ double tile[];
  const int64_t e0 = int64_t(blockIdx.x) * epc;
  const int ecount = int(ne - e0 < epc ? ne - e0 : epc);
  const int n = ecount * nb * nv;
  const double* src = pts + e0 * nb * nv;
  for (int i = threadIdx.x; i < n; i += blockDim.x) tile[i] = src[i];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int le = i / (nv * nb), r = i - le * nv * nb, v = r / nb, b = r - v * nb;
    st[(e0 + le) * ustride + v * nb + b] = tile[(le * nb + b) * nv + v];
  }
}

// Copy n doubles from host memory the device maps (pinned) to device memory: a grid-stride loop, eight loads
// in flight per thread, so that a small grid (one narrow CTA per SM) keeps the CPU-GPU link busy beside other
// kernels while taking few of their registers and warp slots.
__global__ void __launch_bounds__(128) hostCopyKernel(const double* __restrict__ src, double* __restrict__ dst,
                                                      int64_t n) {
  constexpr int kInFlight = 8;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + (kInFlight - 1) * stride < n; i += kInFlight * stride) {
    double v[kInFlight];
#pragma unroll
    for (int k = 0; k < kInFlight; ++k) v[k] = src[i + k * stride];
#pragma unroll
    for (int k = 0; k < kInFlight; ++k) dst[i + k * stride] = v[k];
  }
  for (; i < n; i += stride) dst[i] = src[i];
}

// The same copy into a tensor block's state layout: point-layout element e's value (q, v) (the nodes are the
// points) goes to dst[e * ustride + v * nb + q].  The writes of a warp fall within a few elements' contiguous
// state, which L2 merges before HBM.
__global__ void __launch_bounds__(128) hostCopyTensorKernel(const double* __restrict__ src, double* __restrict__ dst,
                                                            int64_t ne, int nb, int nv, int ustride) {
  constexpr int kInFlight = 8;
  const int64_t n = ne * nb * nv, stride = int64_t(gridDim.x) * blockDim.x;
  const int per = nb * nv;
  const auto target = [&](int64_t i) {
    const int64_t e = i / per;
    const int r = int(i - e * per), q = r / nv, v = r - q * nv;
    return e * ustride + v * nb + q;
  };
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + (kInFlight - 1) * stride < n; i += kInFlight * stride) {
    double x[kInFlight];
#pragma unroll
    for (int k = 0; k < kInFlight; ++k) x[k] = src[i + k * stride];
#pragma unroll
    for (int k = 0; k < kInFlight; ++k) dst[target(i + k * stride)] = x[k];
  }
  for (; i < n; i += stride) dst[target(i)] = src[i];
}

__global__ void stateToPointsTiledKernel(const double* __restrict__ st, double* __restrict__ pts,
                                         const double* __restrict__ phi, int64_t ne, int nb, int nq, int nv,
                                         int ustride, int epc) {
  extern __shared__ double tile[];
  const int64_t e0 = int64_t(blockIdx.x) * epc;
  const int ecount = int(ne - e0 < epc ? ne - e0 : epc);
  const int n = ecount * nq * nv;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int le = i / (nv * nq), r = i - le * nv * nq, v = r / nq, q = r - v * nq;
    const double* u = st + (e0 + le) * ustride + v * nb;
    double s;
    if (!phi) s = u[q];
    else { s = 0.0; for (int b = 0; b < nb; ++b) s = fma(phi[q * nb + b], u[b], s); }
    tile[(le * nq + q) * nv + v] = s;
  }
  __syncthreads();
  double* dst = pts + e0 * nq * nv;
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = tile[i];
}

// Transposes of the two conversions on dense blocks, for cotangents: st = Phi^T pts (of stateToPoint) and
// pts = P^T st (of pointToState, P the least-squares projection [nb][nq]).
__global__ void phiTransposeKernel(const double* __restrict__ pts, double* __restrict__ st, const double* __restrict__ phi,
                                   int64_t ne, int nb, int nq, int nv, int ustride) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ne * nb) return;
  const int64_t e = t / nb;
  const int b = int(t - e * nb);
  for (int v = 0; v < nv; ++v) {
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s = fma(phi[q * nb + b], pts[(e * nq + q) * nv + v], s);
    st[e * ustride + v * nb + b] = s;
  }
}

__global__ void projTransposeKernel(const double* __restrict__ st, double* __restrict__ pts, const double* __restrict__ proj,
                                    int64_t ne, int nb, int nq, int nv, int ustride) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ne * nq) return;
  const int64_t e = t / nq;
  const int q = int(t - e * nq);
  for (int v = 0; v < nv; ++v) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s = fma(proj[b * nq + q], st[e * ustride + v * nb + b], s);
    pts[(e * nq + q) * nv + v] = s;
  }
}

// (rho, u, T) -> (rho, rho u, rho E) in place (VariableConvertor.cpp:341-366).
__global__ void primitiveToConservedKernel(double* __restrict__ pts, int64_t n, int dim, Phys ph) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double* p = pts + t * (dim + 2);
  const double rho = p[0];
  double u2 = 0.0;
  for (int k = 0; k < dim; ++k) { u2 += p[1 + k] * p[1 + k]; p[1 + k] *= rho; }
  // incompressible: rho e with e = cv T (VariableConvertor.cpp:354-362)
  p[dim + 1] = ph.incomp ? rho * (ph.cv * p[dim + 1]) : rho * (ph.cv * p[dim + 1] + u2 / 2.0);
}

// dt = min CFL*minEdge/((|u|+c)(P+1)^2) over points (TimeIntegration.cpp:104-131); per-CTA minima.
__global__ void deltaTimeKernel(const double* __restrict__ pts, const double* __restrict__ minEdge, int64_t n, int nq,
                                int dim, double cfl, double p1sq, Phys ph, double* __restrict__ part) {
  __shared__ double sh[256];
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double dt = 1.79769313486231570e308;
  if (t < n) {
    const double* p = pts + t * (dim + 2);
    const double rho = p[0];
    double u2 = 0.0;
    for (int k = 0; k < dim; ++k) { const double u = p[1 + k] / rho; u2 += u * u; }
    const double e = p[dim + 1] / rho - u2 / 2.0;
    const double pr = ph.gm1 * rho * e;
    const double c = ph.incomp ? ph.c0 : sqrt(ph.gamma * pr / rho);
    dt = cfl * minEdge[t / nq] / ((sqrt(u2) + c) * p1sq);
  }
  sh[threadIdx.x] = dt;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = fmin(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}


}  // namespace sdg

namespace {
thread_local std::string g_create_error;
}  // namespace

namespace sdg {
void setCreateError(const std::string& message) { g_create_error = message; }
}  // namespace sdg

namespace {

using namespace sdg;

template <typename T>
T* devAlloc(size_t count) {
  T* p = nullptr;
  if (count == 0) count = 1;
  SDG_CUDA(cudaMalloc(&p, count * sizeof(T)));
  return p;
}
template <typename T>
void upload(T* dst, const std::vector<T>& src, cudaStream_t s) {
  if (!src.empty()) SDG_CUDA(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

void dropTimingEvents(sdg_handle* h) {
  for (auto& ev : h->timedEvents) { cudaEventDestroy(ev[0]); cudaEventDestroy(ev[1]); }
  h->timedEvents.clear();
  h->timedClass.clear();
}

// Optional event bracketing of each launch (diagnostic kernel timing).
void beginLaunch(sdg_handle* h, int cls, cudaStream_t s) {
  if (!h->timing) return;
  std::array<cudaEvent_t, 2> ev;
  SDG_CUDA(cudaEventCreate(&ev[0]));
  SDG_CUDA(cudaEventCreate(&ev[1]));
  SDG_CUDA(cudaEventRecord(ev[0], s));
  h->timedEvents.push_back(ev);
  h->timedClass.push_back(cls);
}

void checkLaunch(sdg_handle* h, cudaStream_t s) {
  h->launches++;
  SDG_CUDA(cudaGetLastError());
  if (h->timing && !h->timedEvents.empty()) SDG_CUDA(cudaEventRecord(h->timedEvents.back()[1], s));
}
void checkLaunch(sdg_handle* h) { checkLaunch(h, h->stream); }

// ---- geometry --------------------------------------------------------------------------------------
void shapeGrad(int type, const double* X, double* N, double* G /* [nv][3] */) {
  const int nv = typeVertices(type);
  if (type == SDG_ELEMENT_LINE) {
    N[0] = 0.5 * (1 - X[0]); N[1] = 0.5 * (1 + X[0]);
    const double g[6] = {-0.5, 0, 0, 0.5, 0, 0};
    std::copy(g, g + 6, G);
    return;
  }
  if (type == SDG_ELEMENT_TRIANGLE) {
    N[0] = 1 - X[0] - X[1]; N[1] = X[0]; N[2] = X[1];
    const double g[9] = {-1, -1, 0, 1, 0, 0, 0, 1, 0};
    std::copy(g, g + 9, G);
    return;
  }
  if (type == SDG_ELEMENT_TETRAHEDRON) {
    N[0] = 1 - X[0] - X[1] - X[2]; N[1] = X[0]; N[2] = X[1]; N[3] = X[2];
    const double g[12] = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::copy(g, g + 12, G);
    return;
  }
  for (int v = 0; v < nv; ++v) {
    double R[3]; referenceVertex(type, v, R);
    const double a = 1 + R[0] * X[0], b = 1 + R[1] * X[1];
    if (type == SDG_ELEMENT_QUADRANGLE) {
      N[v] = 0.25 * a * b; G[v * 3] = 0.25 * R[0] * b; G[v * 3 + 1] = 0.25 * a * R[1]; G[v * 3 + 2] = 0;
    } else {
      const double c = 1 + R[2] * X[2];
      N[v] = 0.125 * a * b * c;
      G[v * 3] = 0.125 * R[0] * b * c; G[v * 3 + 1] = 0.125 * a * R[1] * c; G[v * 3 + 2] = 0.125 * a * b * R[2];
    }
  }
}

// Jacobian J[l][k] = dx_l/dxi_k at reference point X, physical point x.
void jacobianAt(int type, int dim, const double* nodes, const int32_t* vv, const double* X, double J[3][3], double* x) {
  double N[8], G[24];
  shapeGrad(type, X, N, G);
  for (int l = 0; l < 3; ++l) { x[l] = 0; for (int k = 0; k < 3; ++k) J[l][k] = 0; }
  for (int v = 0; v < typeVertices(type); ++v) {
    const double* c = &nodes[size_t(vv[v]) * 3];
    for (int l = 0; l < 3; ++l) x[l] += N[v] * c[l];
    for (int l = 0; l < dim; ++l)
      for (int k = 0; k < dim; ++k) J[l][k] += G[v * 3 + k] * c[l];
  }
}

// |J| J^-1 (adjugate, row b = |J| dxi_b/dx) and det.
double adjugate(int dim, const double J[3][3], double A[3][3]) {
  if (dim == 1) { A[0][0] = 1.0; return J[0][0]; }
  if (dim == 2) {
    A[0][0] = J[1][1]; A[0][1] = -J[0][1]; A[1][0] = -J[1][0]; A[1][1] = J[0][0];
    return J[0][0] * J[1][1] - J[0][1] * J[1][0];
  }
  A[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  A[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  A[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  A[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  A[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  A[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  A[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  A[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  A[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * A[0][0] + J[0][1] * A[1][0] + J[0][2] * A[2][0];
}

bool isAffine(int type, const double* nodes, const int32_t* vv, double tol) {
  if (type == SDG_ELEMENT_TRIANGLE || type == SDG_ELEMENT_LINE || type == SDG_ELEMENT_TETRAHEDRON) return true;
  const auto P = [&](int k, int d) { return nodes[size_t(vv[k]) * 3 + d]; };
  for (int d = 0; d < 3; ++d) {
    if (type == SDG_ELEMENT_QUADRANGLE) {
      if (std::fabs(P(0, d) + P(2, d) - P(1, d) - P(3, d)) > tol) return false;
    } else {
      const double o = P(0, d), a = P(1, d) - o, b = P(3, d) - o, c = P(4, d) - o;
      if (std::fabs(P(2, d) - (o + a + b)) > tol || std::fabs(P(5, d) - (o + a + c)) > tol ||
          std::fabs(P(7, d) - (o + b + c)) > tol || std::fabs(P(6, d) - (o + a + b + c)) > tol)
        return false;
    }
  }
  return true;
}

double minEdgeOf(int type, const double* nodes, const int32_t* vv) {
  static const int lineE[1][2] = {{0, 1}};
  static const int triE[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  static const int quadE[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
  static const int hexE[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6}, {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
  static const int tetE[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 2}, {3, 1}};
  const int(*E)[2] = type == SDG_ELEMENT_LINE ? lineE
                     : (type == SDG_ELEMENT_TRIANGLE ? triE
                        : (type == SDG_ELEMENT_QUADRANGLE ? quadE : (type == SDG_ELEMENT_TETRAHEDRON ? tetE : hexE)));
  const int nE = type == SDG_ELEMENT_LINE ? 1
                 : (type == SDG_ELEMENT_TRIANGLE ? 3
                    : (type == SDG_ELEMENT_QUADRANGLE ? 4 : (type == SDG_ELEMENT_TETRAHEDRON ? 6 : 12)));
  double best = 1e300;
  for (int i = 0; i < nE; ++i) {
    double s = 0;
    for (int d = 0; d < 3; ++d) { const double t = nodes[size_t(vv[E[i][0]]) * 3 + d] - nodes[size_t(vv[E[i][1]]) * 3 + d]; s += t * t; }
    best = std::min(best, std::sqrt(s));
  }
  return best;
}

// ---- tensor tables ---------------------------------------------------------------------------------
void buildTensorTables(DevBlock& B) {
  TensorTables T;
  std::memset(&T, 0, sizeof(T));
  const TensorOps& o = B.ops;
  const int n = o.n, dim = B.dim;
  for (int a = 0; a < n; ++a) {
    for (int i = 0; i < n; ++i) { T.dhat[a][i] = o.dhat[a][i]; T.b1[a][i] = o.b1[a][i]; }
    T.endm[a] = o.endm[a]; T.endp[a] = o.endp[a]; T.liftm[a] = o.liftm[a]; T.liftp[a] = o.liftp[a]; T.w[a] = o.w[a];
  }
  const PointRule fr = faceRule(B.type, B.p);
  const auto gaussIndex = [&](double t) {
    for (int g = 0; g < n; ++g) if (std::fabs(o.x[g] - t) < 1e-12) return g;
    throw Failure(SDG_ERR_INVALID_ARGUMENT, "face point does not lie on a Gauss line");
  };
  const int stride[3] = {dim == 1 ? 1 : (dim == 2 ? n : n * n), dim == 2 ? 1 : n, 1};
  for (int f = 0; f < B.nface; ++f) {
    int axis = -1, end = 0;
    for (int j = 0; j < B.nfq; ++j) {
      double X[3]; facePointInParent(B.type, f, &fr.x[j * 3], X);
      int idx[3] = {0, 0, 0};
      int ax = -1;
      for (int d = 0; d < dim; ++d) {
        if (std::fabs(std::fabs(X[d]) - 1.0) < 1e-12) { ax = d; end = X[d] > 0 ? 1 : 0; idx[d] = 0; }
        else idx[d] = gaussIndex(X[d]);
      }
      if (ax < 0 || (axis >= 0 && ax != axis)) throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad face table");
      axis = ax;
      int base = 0;
      for (int d = 0; d < dim; ++d) base += idx[d] * stride[d];
      T.faceBase[f][j] = base;
      for (int q = 0; q < n; ++q) T.nodeFacePoint[axis][end][base + q * stride[axis]] = (unsigned char)j;
    }
    T.faceAxis[f] = axis; T.faceEnd[f] = end; T.axisFace[axis][end] = f;
  }
  B.tablesHost.assign(sizeof(TensorTables) / 8, 0.0);
  std::memcpy(B.tablesHost.data(), &T, sizeof(T));
}

}  // namespace

namespace sdg {

// ---- kernel configuration ---------------------------------------------------------------------------
namespace {
std::mutex g_kernel_mutex;
std::set<std::pair<int, const void*>> g_configured;
std::map<int, int> g_optin, g_sms;
}  // namespace

int sharedMemoryOptin(int device) {
  std::lock_guard<std::mutex> lock(g_kernel_mutex);
  auto it = g_optin.find(device);
  if (it != g_optin.end()) return it->second;
  int v = 0;
  SDG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  g_optin[device] = v;
  return v;
}

int multiprocessorCount(int device) {
  std::lock_guard<std::mutex> lock(g_kernel_mutex);
  auto it = g_sms.find(device);
  if (it != g_sms.end()) return it->second;
  int v = 0;
  SDG_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device));
  g_sms[device] = v;
  return v;
}

void configureKernel(const void* fn, int device) {
  if (!fn) return;
  const int optin = sharedMemoryOptin(device);
  std::lock_guard<std::mutex> lock(g_kernel_mutex);
  if (!g_configured.insert({device, fn}).second) return;
  SDG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
}

void setStageTile(DevBlock& B, int slot, int epb, int threads) {
  const KernelVariant& v = B.stageV[slot];
  B.epb = epb;
  B.threads = v.nodeThreads ? v.threadsFor(epb) : threads;
  B.smem = v.smem(B.epb, B.threads);
  B.grid = (B.ne + epb - 1) / epb;
}

void setGradTile(DevBlock& B, int epb, int threads) {
  B.gepb = epb;
  B.gthreads = B.gradV.nodeThreads ? B.gradV.threadsFor(epb) : threads;
  B.gsmem = B.gradV.smem(B.gepb, B.gthreads);
  B.ggrid = (B.ne + epb - 1) / epb;
}

namespace {

// Kernel variants of a block (element kind, order, affine) and its default tiles.
void resolveBlock(DevBlock& B, int slot, bool br2) {
  for (int visc = 0; visc < 3; ++visc)
    B.stageV[visc] = B.kind == kTensor ? tensorStageVariant(B.dim, B.n, B.affine != 0, visc)
                                       : denseStageVariant(B.type, B.p, B.affine != 0, visc);
  B.gradV = B.kind == kTensor ? tensorGradVariant(B.dim, B.n, B.affine != 0, br2)
                              : denseGradVariant(B.type, B.p, B.affine != 0);
  // the variant of the block's equations must exist (tetrahedra: the Euler stage only)
  if (!B.stageV[slot].valid() || (slot > 0 && !B.gradV.valid()))
    throw Failure(SDG_ERR_UNSUPPORTED, "unsupported element block (type, order, affine)");
  const KernelVariant& v = B.stageV[slot];
  B.ustride = ((B.dim + 2) * B.nb + 1) & ~1;
  B.fstride = B.nface * (B.dim + 2) * B.nfq;
  setStageTile(B, slot, v.epb, v.threads);
  setGradTile(B, B.gradV.epb, B.gradV.threads);
}

}  // namespace

// ---- launch records ---------------------------------------------------------------------------------
Rec stageRec(sdg_handle* h, DevBlock& B) {
  Rec r;
  r.kind = kRecStage; r.cls = 0;
  const KernelVariant& v = B.stageV[stageSlot(h)];
  r.fn = v.single; r.bfn = v.batch;
  r.threads = B.threads; r.epb = B.epb; r.smem = B.smem; r.units = B.grid;
  StageArgs& a = r.sa;
  std::memset(&a, 0, sizeof(a));
  a.face = h->face; a.geom = B.geom; a.tables = B.tables; a.status = h->status;
  a.ne = B.ne; a.faceBase = B.faceBase; a.epb = B.epb;
  a.txExtra = h->txExtra; a.waitLimit = h->waitLimit; a.diagMetric = B.diagMetric;
  if (viscousPath(h)) { a.fluxSrc = h->faceFlux; a.grad = h->grad + B.gradOffset; }
  if (h->av) { a.av = 1; a.epsV = B.epsV; a.avTab = B.avTab; }
  r.ph = h->ph;
  return r;
}

Rec gradRec(sdg_handle* h, DevBlock& B, int which) {
  Rec r;
  r.cls = 4;
  r.fn = B.gradV.single; r.bfn = B.gradV.batch;
  r.threads = B.gthreads; r.epb = B.gepb; r.smem = B.gsmem; r.units = B.ggrid;
  const double* u = h->state[which] ? h->state[which] + B.stateOffset : nullptr;
  double* g = h->grad ? h->grad + B.gradOffset : nullptr;
  // artificial viscosity runs the BR2 layout (own and neighbour traces, the volume gradient)
  const int br2 = h->cfg.viscous_flux == SDG_VISCOUS_BR2 || h->av;
  if (B.kind == kTensor) {
    r.kind = kRecGradTensor;
    GradArgs& a = r.ga;
    std::memset(&a, 0, sizeof(a));
    a.u = u; a.face = h->face; a.faceOther = h->faceOther; a.faceGrad = h->faceGrad; a.grad = g;
    a.geom = B.geom; a.fmetric = B.fmetric; a.fmetricPoint = B.facePoint; a.tables = B.tables; a.status = h->status;
    a.ne = B.ne; a.faceBase = B.faceBase; a.br2 = br2; a.epb = B.gepb;
    if (h->av) { a.av = 1; a.epsV = B.epsV; a.avTab = B.avTab; }
  } else {
    r.kind = kRecGradDense;
    DenseGradArgs& a = r.da;
    std::memset(&a, 0, sizeof(a));
    a.u = u; a.face = h->face; a.faceOther = h->faceOther; a.faceGrad = h->faceGrad; a.grad = g;
    a.geom = B.geom; a.fmetric = B.fmetric; a.fmetricPoint = B.facePoint; a.tables = B.tables; a.status = h->status;
    a.ne = B.ne; a.faceBase = B.faceBase; a.br2 = br2; a.epb = B.gepb;
    if (h->av) { a.av = 1; a.epsV = B.epsV; a.avTab = B.avTab; }
  }
  return r;
}

namespace {
bool boundaryOp(int op) {
  return op == kOpFaceBoundary || op == kOpExchangeBoundary || op == kOpFaceNSBoundary || op == kOpFaceAVBoundary;
}
}  // namespace

Rec faceRec(sdg_handle* h, int op) {
  Rec r;
  r.kind = kRecFace;
  const bool bnd = boundaryOp(op);
  r.cls = bnd ? 2 : 1;
  r.fn = h->faceV[op].single; r.bfn = h->faceV[op].batch;
  r.threads = kFaceThreads; r.epb = 1; r.smem = 0;
  FaceArgs& f = r.fa;
  std::memset(&f, 0, sizeof(f));
  f.face = h->face; f.other = h->faceOther; f.faceGrad = h->faceGrad; f.faceFlux = h->faceFlux;
  f.conn = bnd ? h->bconn : h->fconn; f.fgeo = bnd ? h->bgeo : h->fgeo; f.ghost = h->ghost;
  f.nface = bnd ? h->nBoundary : h->nInterior; f.n1d = h->n1d; f.ph = h->ph; f.perm = h->facePerm;
  f.fgeoPoint = h->facePoint ? 1 : 0;
  const int64_t points = f.nface * h->nfq;
  r.units = (points + kFaceThreads - 1) / kFaceThreads;
  // one thread per face point does a whole Riemann flux in FP64: with fewer points than two full CTAs per SM,
  // narrower CTAs spread them over every SM instead of leaving most SMs idle (one-instance launches only)
  const int64_t sms = h->hostOnly ? 0 : multiprocessorCount(h->device);
  if (points > 0 && points < sms * 2 * kFaceThreads) {
    const int64_t t = std::min<int64_t>(kFaceThreads, std::max<int64_t>(32, ((points + 2 * sms - 1) / (2 * sms) + 31) / 32 * 32));
    r.soloThreads = int(t);
    r.soloUnits = (points + t - 1) / t;
  }
  return r;
}

namespace {

Rec relRec(sdg_handle* h) {
  Rec r;
  r.kind = kRecRelerr; r.cls = 3;
  const KernelVariant v = relerrVariant();
  r.fn = v.single; r.bfn = v.batch;
  r.threads = 256; r.epb = 1; r.smem = 0; r.units = h->nv;
  RelArgs& a = r.ra;
  std::memset(&a, 0, sizeof(a));
  a.part = h->relPart; a.out = h->relOut; a.inv_elements = 1.0 / double(h->elements); a.nv = h->nv;
  a.nranges = int(h->blocks.size());
  for (size_t b = 0; b < h->blocks.size(); ++b) { a.offset[b] = h->blocks[b].relOffset; a.count[b] = h->blocks[b].grid; }
  return r;
}

}  // namespace

const double kRk[3][3][3] = {{{1.0, 0.0, 1.0}, {0, 0, 0}, {0, 0, 0}},
                             {{1.0, 0.0, 1.0}, {0.5, 0.5, 0.5}, {0, 0, 0}},
                             {{1.0, 0.0, 1.0}, {0.75, 0.25, 0.25}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}}};  // TimeIntegration.cpp:45-65

namespace {

// Face fluxes of the state in buffer `which` (whose traces the face buffer holds): NS gradient pass first.
void emitFluxes(sdg_handle* h, int which, int seq, std::vector<Rec>& out) {
  const auto push = [&](Rec r, int level) { r.seq = seq + level; out.push_back(r); };
  if (viscousPath(h)) {
    if (h->nInterior > 0) push(faceRec(h, kOpExchange), 0);
    if (h->nBoundary > 0) push(faceRec(h, kOpExchangeBoundary), 0);
    for (DevBlock& B : h->blocks) push(gradRec(h, B, which), 1);
    if (h->nInterior > 0) push(faceRec(h, h->av ? kOpFaceAV : kOpFaceNS), 2);
    if (h->nBoundary > 0) push(faceRec(h, h->av ? kOpFaceAVBoundary : kOpFaceNSBoundary), 2);
  } else {
    if (h->nInterior > 0) push(faceRec(h, kOpFace), 2);
    if (h->nBoundary > 0) push(faceRec(h, kOpFaceBoundary), 2);
  }
}

}  // namespace

// One full RK step; state[0] holds U^n on entry and U^{n+1} on exit, the face buffer holds its traces.
// Stage s: fluxes of its input, then per block volume + lift + update + new traces (TimeIntegration.cpp:326-350).
void emitStep(sdg_handle* h, double dt, bool relerr, std::vector<Rec>& out) {
  const int ns = h->cfg.time_integration + 1;
  // artificial viscosity of the step's initial state, once per step (TimeIntegration.cpp:336-338); its
  // three dependent levels sit before stage 0's (-3, -2, -1)
  if (h->av) emitArtificialViscosity(h, -3, out);
  for (int s = 0; s < ns; ++s) {
    emitFluxes(h, s == 0 ? 0 : 1, s * 8, out);
    const bool last = s == ns - 1;
    for (DevBlock& B : h->blocks) {
      Rec r = stageRec(h, B);
      StageArgs& a = r.sa;
      a.uin = h->state[s == 0 ? 0 : 1] + B.stateOffset;
      a.ubase = h->state[0] + B.stateOffset;
      a.uout = h->state[last ? 0 : 1] + B.stateOffset;
      a.c0 = kRk[h->cfg.time_integration][s][0];
      a.c1 = kRk[h->cfg.time_integration][s][1];
      a.c2dt = kRk[h->cfg.time_integration][s][2] * dt;
      a.doUpdate = 1; a.doTrace = 1; a.doVolume = 1;
      a.relerr = (relerr && last) ? h->relPart + B.relOffset * h->nv : nullptr;
      if (last && h->pointsOut && B.kind == kTensor) a.pointsOut = h->pointsOut + B.pointOffset * h->nv;
      r.seq = s * 8 + 3;
      out.push_back(r);
    }
  }
  if (relerr) {
    Rec r = relRec(h);
    r.seq = 8 * ns;
    out.push_back(r);
  }
}

namespace {

void launchOne(const Rec& r, cudaStream_t s) {
  void* p[2];
  switch (r.kind) {
    case kRecStage: p[0] = const_cast<StageArgs*>(&r.sa); p[1] = const_cast<Phys*>(&r.ph); break;
    case kRecGradTensor: p[0] = const_cast<GradArgs*>(&r.ga); break;
    case kRecGradDense: p[0] = const_cast<DenseGradArgs*>(&r.da); break;
    case kRecFace: p[0] = const_cast<FaceArgs*>(&r.fa); break;
    case kRecAv: p[0] = const_cast<AvArgs*>(&r.av); break;
    default: p[0] = const_cast<RelArgs*>(&r.ra); break;
  }
  if (r.units <= 0) return;
  const int64_t units = r.soloThreads ? r.soloUnits : r.units;
  const int threads = r.soloThreads ? r.soloThreads : r.threads;
  if (units > 0x7fffffffLL) throw Failure(SDG_ERR_UNSUPPORTED, "launch exceeds the grid limit");
  SDG_CUDA(cudaLaunchKernel(r.fn, dim3(unsigned(units)), dim3(unsigned(threads)), p, r.smem, s));
}

}  // namespace

void runRecs(sdg_handle* h, const std::vector<Rec>& recs, cudaStream_t stream) {
  for (const Rec& r : recs) {
    if (r.units <= 0) continue;
    beginLaunch(h, r.cls, stream);
    launchOne(r, stream);
    checkLaunch(h, stream);
  }
}

void dropGraph(sdg_handle* h) {
  if (h->graphExec) cudaGraphExecDestroy(h->graphExec);
  h->graphExec = nullptr;
  h->graphKernels = 0;
}

// Face traces of state buffer `which` (initial condition or after a state upload).
void traceAll(sdg_handle* h, int which) {
  std::vector<Rec> recs;
  for (DevBlock& B : h->blocks) {
    Rec r = stageRec(h, B);
    r.sa.uin = h->state[which] + B.stateOffset;
    r.sa.doTrace = 1; r.sa.doVolume = 0; r.sa.doUpdate = 0;
    recs.push_back(r);
  }
  runRecs(h, recs, h->stream);
}

void checkStatus(sdg_handle* h) {
  unsigned st = 0;
  SDG_CUDA(cudaMemcpyAsync(&st, h->status, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  if (st & kStatusTimeout) throw Failure(SDG_ERR_TIMEOUT, "a bounded device wait timed out");
}

namespace {

// One step through a captured CUDA graph (re-captured when dt or the tiles change).
void stepGraph(sdg_handle* h, double dt) {
  if (!h->graphExec || h->graphDt != dt || h->graphOut != h->pointsOut) {
    dropGraph(h);
    std::vector<Rec> recs;
    emitStep(h, dt, true, recs);
    cudaGraph_t graph = nullptr;
    SDG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    try {
      for (const Rec& r : recs) launchOne(r, h->stream);
    } catch (...) {
      cudaStreamEndCapture(h->stream, &graph);
      if (graph) cudaGraphDestroy(graph);
      throw;
    }
    SDG_CUDA(cudaStreamEndCapture(h->stream, &graph));
    const cudaError_t e = cudaGraphInstantiate(&h->graphExec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { h->graphExec = nullptr; SDG_CUDA(e); }
    h->graphDt = dt;
    h->graphOut = h->pointsOut;
    h->graphKernels = 0;
    for (const Rec& r : recs) h->graphKernels += r.units > 0;
  }
  SDG_CUDA(cudaGraphLaunch(h->graphExec, h->stream));
  h->launches += h->graphKernels;
}

void stepOnce(sdg_handle* h, double dt) {
  h->gradInput = stepGradientInput(h);
  if (h->useGraph && !h->timing) { stepGraph(h, dt); return; }
  std::vector<Rec> recs;
  emitStep(h, dt, true, recs);
  runRecs(h, recs, h->stream);
}

int fail(sdg_handle* h, const Failure& f) {
  if (h) h->err = f.what();
  else g_create_error = f.what();
  return f.code;
}

#define SDG_API_BEGIN try {
#define SDG_API_END(h)                                             \
  }                                                                \
  catch (const Failure& f) { return fail(h, f); }                  \
  catch (const std::exception& ex) { return fail(h, Failure(SDG_ERR_INVALID_ARGUMENT, ex.what())); }


// Convert a point-layout array in h->scratch to the state buffer `which` (tensor: transpose; dense:
// unweighted least-squares projection, InitialCondition.cpp:91-104).
// The host buffer itself when it is pinned host memory the device reaches at the same address (page-locked
// and mapped, as every cudaHostAlloc / cudaHostRegister allocation is under unified addressing), else null.
const double* mappedHost(const double* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost && at.devicePointer == static_cast<const void*>(p) ? p : nullptr;
}

// Elements per CTA of the tiled conversions: the tile ([elements][nq][nv] doubles) within 48 KB.
int conversionElements(const DevBlock& B, int nv) {
  const int per = B.nq * nv;
  return per > 6144 ? 1 : 6144 / per;
}

// Conserved variables at the volume points (point layout) -> state[which].  A pinned host buffer is read in
// place over the CPU-GPU link on tensor blocks (one pass: transfer and transpose together); otherwise, and on
// dense blocks (whose least-squares projection re-reads each point), the block's points are first copied to
// the scratch buffer.
void uploadPoints(sdg_handle* h, const double* conserved, int which) {
  const double* mapped = mappedHost(conserved);
  for (DevBlock& B : h->blocks) {
    const size_t off = B.pointOffset * h->nv, count = size_t(B.ne) * B.nq * h->nv;
    if (mapped && B.kind == kTensor) {
      const int epc = conversionElements(B, h->nv);
      const int64_t grid = (B.ne + epc - 1) / epc;
      pointsToTensorStateKernel<<<unsigned(grid), 256, size_t(epc) * B.nq * h->nv * 8, h->stream>>>(
          mapped + off, h->state[which] + B.stateOffset, B.ne, B.nb, h->nv, B.ustride, epc);
    } else {
      SDG_CUDA(cudaMemcpyAsync(h->scratch + off, conserved + off, count * 8, cudaMemcpyHostToDevice, h->stream));
      const int grid = int((B.ne * B.nb + 255) / 256);
      pointToStateKernel<<<grid, 256, 0, h->stream>>>(h->scratch + off, h->state[which] + B.stateOffset,
                                                      B.kind == kDense ? B.lsqDev : nullptr, B.ne, B.nb, B.nq, h->nv,
                                                      B.ustride);
    }
    checkLaunch(h);
  }
}

// state[which] -> conserved variables at the volume points in a host buffer: written in place over the link
// when it is pinned, else through the scratch buffer and one copy.  skipTensor (pinned buffers only): the
// tensor blocks' points are already there (written by the step's last stage).
void downloadPoints(sdg_handle* h, int which, double* conserved, bool skipTensor = false) {
  double* mapped = const_cast<double*>(mappedHost(conserved));
  double* dst = mapped ? mapped : h->scratch;
  for (DevBlock& B : h->blocks) {
    if (mapped && skipTensor && B.kind == kTensor) continue;
    const int epc = conversionElements(B, h->nv);
    const int64_t grid = (B.ne + epc - 1) / epc;
    stateToPointsTiledKernel<<<unsigned(grid), 256, size_t(epc) * B.nq * h->nv * 8, h->stream>>>(
        h->state[which] + B.stateOffset, dst + B.pointOffset * h->nv, B.kind == kDense ? B.phiDev : nullptr, B.ne,
        B.nb, B.nq, h->nv, B.ustride, epc);
    checkLaunch(h);
  }
  if (!mapped)
    SDG_CUDA(cudaMemcpyAsync(conserved, h->scratch, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyDeviceToHost,
                             h->stream));
}

// Point-layout device array `src` (default: the scratch buffer) -> state[which].
void pointsToState(sdg_handle* h, int which, const double* src = nullptr) {
  if (!src) src = h->scratch;
  for (DevBlock& B : h->blocks) {
    const int64_t work = B.ne * (B.kind == kTensor ? B.nb : B.nb);
    const int grid = int((work + 255) / 256);
    pointToStateKernel<<<grid, 256, 0, h->stream>>>(src + B.pointOffset * h->nv, h->state[which] + B.stateOffset,
                                                    B.kind == kDense ? B.lsqDev : nullptr, B.ne, B.nb, B.nq, h->nv,
                                                    B.ustride);
    checkLaunch(h);
  }
}
}  // namespace

void pointsToStateBuffer(sdg_handle* h, const double* pts, double* st) {
  for (DevBlock& B : h->blocks) {
    const int grid = int((B.ne * B.nb + 255) / 256);
    pointToStateKernel<<<grid, 256, 0, h->stream>>>(pts + B.pointOffset * h->nv, st + B.stateOffset,
                                                    B.kind == kDense ? B.lsqDev : nullptr, B.ne, B.nb, B.nq, h->nv,
                                                    B.ustride);
    checkLaunch(h);
  }
}

// Cotangents: the transposes of stateToPointsBuffer (points -> state) and of pointsToStateBuffer (state ->
// points).  On tensor blocks both maps are the same permutation of the layout, whose transpose is its inverse.
void cotangentPointsToState(sdg_handle* h, const double* pts, double* st) {
  for (DevBlock& B : h->blocks) {
    const int grid = int((B.ne * B.nb + 255) / 256);
    if (B.kind == kDense)
      phiTransposeKernel<<<grid, 256, 0, h->stream>>>(pts + B.pointOffset * h->nv, st + B.stateOffset, B.phiDev, B.ne,
                                                      B.nb, B.nq, h->nv, B.ustride);
    else
      pointToStateKernel<<<grid, 256, 0, h->stream>>>(pts + B.pointOffset * h->nv, st + B.stateOffset, nullptr, B.ne,
                                                      B.nb, B.nq, h->nv, B.ustride);
    checkLaunch(h);
  }
}

void cotangentStateToPoints(sdg_handle* h, const double* st, double* pts) {
  for (DevBlock& B : h->blocks) {
    const int grid = int((B.ne * B.nq + 255) / 256);
    if (B.kind == kDense)
      projTransposeKernel<<<grid, 256, 0, h->stream>>>(st + B.stateOffset, pts + B.pointOffset * h->nv, B.lsqDev, B.ne,
                                                       B.nb, B.nq, h->nv, B.ustride);
    else
      stateToPointKernel<<<grid, 256, 0, h->stream>>>(st + B.stateOffset, pts + B.pointOffset * h->nv, nullptr, B.ne,
                                                      B.nb, B.nq, h->nv, B.ustride);
    checkLaunch(h);
  }
}

void stateToPointsBuffer(sdg_handle* h, const double* st, double* pts) {
  for (DevBlock& B : h->blocks) {
    const int grid = int((B.ne * B.nq + 255) / 256);
    stateToPointKernel<<<grid, 256, 0, h->stream>>>(st + B.stateOffset, pts + B.pointOffset * h->nv,
                                                    B.kind == kDense ? B.phiDev : nullptr, B.ne, B.nb, B.nq, h->nv,
                                                    B.ustride);
    checkLaunch(h);
  }
}

namespace {

void stateToPoints(sdg_handle* h, int which) {
  for (DevBlock& B : h->blocks) {
    const int64_t work = B.ne * B.nq;
    const int grid = int((work + 255) / 256);
    stateToPointKernel<<<grid, 256, 0, h->stream>>>(h->state[which] + B.stateOffset, h->scratch + B.pointOffset * h->nv,
                                                    B.kind == kDense ? B.phiDev : nullptr, B.ne, B.nb, B.nq, h->nv,
                                                    B.ustride);
    checkLaunch(h);
  }
}

// Times launch(iters) on the legacy stream, doubling iters until one launch takes at least ms/2, and
// returns flopPerIter(threads * blocks) * iters / time in GFLOP/s.
template <class Launch>
double timeProbe(int device, double ms, double flopsPerIteration, Launch launch) {
  SDG_CUDA(cudaSetDevice(device));
  cudaEvent_t e0, e1;
  SDG_CUDA(cudaEventCreate(&e0));
  SDG_CUDA(cudaEventCreate(&e1));
  int iters = 256;
  float t = 0.f;
  launch(16);
  SDG_CUDA(cudaGetLastError());
  SDG_CUDA(cudaDeviceSynchronize());
  for (int round = 0; round < 12; ++round) {
    SDG_CUDA(cudaEventRecord(e0));
    launch(iters);
    SDG_CUDA(cudaEventRecord(e1));
    SDG_CUDA(cudaEventSynchronize(e1));
    SDG_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (t >= 0.5 * ms || iters >= (1 << 22)) break;
    iters *= 2;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return flopsPerIteration * iters / (double(t) * 1e6);
}

double measureFp64Peak(int device, double ms) {
  SDG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SDG_CUDA(cudaGetDeviceProperties(&prop, device));
  const int threads = 256, blocks = prop.multiProcessorCount * 8;
  double* out = devAlloc<double>(size_t(threads) * blocks);
  const double r = timeProbe(device, ms, 2.0 * 8.0 * double(threads) * blocks, [&](int iters) {
    fp64ProbeKernel<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
  });
  cudaFree(out);
  return r;
}

__global__ void reciprocalProbeKernel(const double* __restrict__ x, double* __restrict__ r, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) r[i] = rcp(x[i]);
}

double measureDmmaPeak(int device, int shape, double ms) {
  SDG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  SDG_CUDA(cudaGetDeviceProperties(&prop, device));
  const int threads = 256, blocks = prop.multiProcessorCount * 8;
  double* out = devAlloc<double>(size_t(threads) * blocks);
  static const int mnk[4][3] = {{8, 8, 4}, {16, 8, 4}, {16, 8, 8}, {16, 8, 16}};
  const double perMma = 2.0 * mnk[shape][0] * mnk[shape][1] * mnk[shape][2];
  const double warps = double(threads / 32) * blocks;
  const double r = timeProbe(device, ms, perMma * 4.0 * warps, [&](int iters) {
    switch (shape) {
      case 0: dmmaProbeKernel<0><<<blocks, threads>>>(out, iters); break;
      case 1: dmmaProbeKernel<1><<<blocks, threads>>>(out, iters); break;
      case 2: dmmaProbeKernel<2><<<blocks, threads>>>(out, iters); break;
      default: dmmaProbeKernel<3><<<blocks, threads>>>(out, iters); break;
    }
  });
  cudaFree(out);
  return r;
}

}  // namespace
}  // namespace sdg

using namespace sdg;

// =====================================================================================================
#pragma GCC visibility push(default)
extern "C" {

const char* sdg_last_error(const sdg_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int sdg_create(const sdg_mesh* mesh, const sdg_config* config, int32_t device, sdg_handle** out) {
  if (!mesh || !config || !out) { g_create_error = "null argument"; return SDG_ERR_INVALID_ARGUMENT; }
  *out = nullptr;
  std::unique_ptr<sdg_handle> H(new sdg_handle());
  sdg_handle* h = H.get();
  try {
    const sdg_config& c = *config;
    if (mesh->dimension < 1 || mesh->dimension > 3) throw Failure(SDG_ERR_INVALID_ARGUMENT, "dimension must be 1, 2 or 3");
    if (c.polynomial_order < 1 || c.polynomial_order > 5) throw Failure(SDG_ERR_INVALID_ARGUMENT, "polynomial order must be 1..5");
    if (c.equation < SDG_COMPRESSIBLE_EULER || c.equation > SDG_INCOMPRESSIBLE_NS) throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad equation");
    const bool incomp = c.equation == SDG_INCOMPRESSIBLE_EULER || c.equation == SDG_INCOMPRESSIBLE_NS;
    const bool viscous = c.equation == SDG_COMPRESSIBLE_NS || c.equation == SDG_INCOMPRESSIBLE_NS;
    if (c.convective_flux < 0 || c.convective_flux > 4) throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad convective flux");
    if (incomp && (c.convective_flux == SDG_FLUX_HLLC || c.convective_flux == SDG_FLUX_ROE))
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "HLLC and Roe need the ideal gas (incompressible models: Central, LF, Exact)");
    if (!incomp && c.convective_flux == SDG_FLUX_EXACT)
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "the Exact flux belongs to the incompressible models");
    if (incomp && (!(c.reference_sound_speed > 0) || !(c.reference_density > 0)))
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "incompressible models need reference_sound_speed and reference_density > 0");
    if (c.source_term != SDG_SOURCE_NONE && c.source_term != SDG_SOURCE_BOUSSINESQ)
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad source term");
    if (c.time_integration < 0 || c.time_integration > 2) throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad time integration");
    if (c.shock_capturing != SDG_SHOCK_NONE && c.shock_capturing != SDG_SHOCK_ARTIFICIAL_VISCOSITY)
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad shock capturing");
    if (c.shock_capturing == SDG_SHOCK_ARTIFICIAL_VISCOSITY) {
      if (!(c.empirical_tolerance > 0) || !(c.artificial_viscosity_factor >= 0))
        throw Failure(SDG_ERR_INVALID_ARGUMENT, "artificial viscosity needs empirical_tolerance > 0 and factor >= 0");
      if (c.equation != SDG_COMPRESSIBLE_EULER)
        throw Failure(SDG_ERR_UNSUPPORTED, "artificial viscosity is built for the compressible Euler equations");
      h->av = true;
    }
    if (!(c.specific_heat_ratio > 1.0) || !(c.specific_heat_constant_volume > 0) || !(c.specific_heat_constant_pressure > 0))
      throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad thermodynamic constants");
    if (viscous) {
      if (c.viscous_flux != SDG_VISCOUS_BR1 && c.viscous_flux != SDG_VISCOUS_BR2)
        throw Failure(SDG_ERR_INVALID_ARGUMENT, "Navier-Stokes needs BR1 or BR2");
      if (!(c.dynamic_viscosity >= 0) || !(c.prandtl_number > 0)) throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad transport constants");
      if (c.transport_model != SDG_TRANSPORT_CONSTANT && c.transport_model != SDG_TRANSPORT_SUTHERLAND)
        throw Failure(SDG_ERR_INVALID_ARGUMENT, "bad transport model");
      h->ns = true;
    }
    if (!mesh->node_coordinate || mesh->node_count <= 0) throw Failure(SDG_ERR_INVALID_ARGUMENT, "no nodes");
    h->cfg = c; h->device = device; h->nodeCount = mesh->node_count;
    h->dim = mesh->dimension; h->nv = h->dim + 2; h->p = c.polynomial_order;
    h->ph.gamma = c.specific_heat_ratio; h->ph.gm1 = c.specific_heat_ratio - 1.0;
    h->ph.cv = c.specific_heat_constant_volume; h->ph.inv_cv = 1.0 / c.specific_heat_constant_volume;
    h->ph.cp = c.specific_heat_constant_pressure; h->ph.mu = c.dynamic_viscosity;
    h->ph.kappa = c.prandtl_number > 0 ? c.specific_heat_constant_pressure * c.dynamic_viscosity / c.prandtl_number : 0.0;
    h->ph.transport = c.transport_model;
    h->ph.hllc_g2 = (c.specific_heat_ratio + 1.0) / (2.0 * c.specific_heat_ratio);
    h->ph.incomp = incomp ? 1 : 0;
    h->ph.c0 = incomp ? c.reference_sound_speed : 0.0;
    h->ph.c02 = h->ph.c0 * h->ph.c0;
    // p = c0^2 (rho - rho0) + 0.01 rho0 c0^2 (calculatePressureAdditionFromSoundSpeedDensity)
    h->ph.rho0 = incomp ? c.reference_density : 0.0;
    h->ph.padd = incomp ? 0.01 * c.reference_density * c.reference_sound_speed * c.reference_sound_speed : 0.0;
    h->ph.source = c.source_term;
    h->ph.beta = c.thermal_expansion_coefficient;
    h->ph.tref = c.reference_temperature;
    // element blocks, in the reference's loop order
    std::vector<Block> mb;
    if (h->dim == 1) {
      if (mesh->line_count > 0) mb.push_back({SDG_ELEMENT_LINE, mesh->line_count, mesh->line_node});
    } else if (h->dim == 2) {
      const int gq = mesh->geometry_order > 1 ? mesh->geometry_order : 1;
      if (mesh->triangle_count > 0)
        mb.push_back({SDG_ELEMENT_TRIANGLE, mesh->triangle_count, mesh->triangle_node,
                      gq > 1 ? mesh->triangle_geometry_node : nullptr, gq});
      if (mesh->quadrangle_count > 0)
        mb.push_back({SDG_ELEMENT_QUADRANGLE, mesh->quadrangle_count, mesh->quadrangle_node,
                      gq > 1 ? mesh->quadrangle_geometry_node : nullptr, gq});
    } else {
      if (mesh->tetrahedron_count > 0 && mesh->hexahedron_count > 0)
        throw Failure(SDG_ERR_UNSUPPORTED, "a mesh of tetrahedra and hexahedra needs pyramids, which are not built");
      if (mesh->tetrahedron_count > 0) {
        mb.push_back({SDG_ELEMENT_TETRAHEDRON, mesh->tetrahedron_count, mesh->tetrahedron_node});
        if (c.polynomial_order > 5) throw Failure(SDG_ERR_UNSUPPORTED, "tetrahedra are built for P = 1..5");
      }
      const int gq = mesh->geometry_order > 1 ? mesh->geometry_order : 1;
      if (mesh->hexahedron_count > 0)
        mb.push_back({SDG_ELEMENT_HEXAHEDRON, mesh->hexahedron_count, mesh->hexahedron_node,
                      gq > 1 ? mesh->hexahedron_geometry_node : nullptr, gq});
    }
    if (mb.empty()) throw Failure(SDG_ERR_INVALID_ARGUMENT, "mesh has no elements of its dimension");
    if (mesh->geometry_order > 1) {
      if (mesh->dimension == 1) throw Failure(SDG_ERR_UNSUPPORTED, "curved (high-order) geometry is built in 2D and 3D");
      if (mesh->dimension == 3 && mesh->tetrahedron_count > 0)
        throw Failure(SDG_ERR_UNSUPPORTED, "curved (high-order) tetrahedra are not built");
      if (mesh->geometry_order > 5) throw Failure(SDG_ERR_INVALID_ARGUMENT, "geometry order must be 1..5");
      for (const Block& b : mb)
        if (!b.geometry) throw Failure(SDG_ERR_INVALID_ARGUMENT, "geometry_order > 1 needs the geometry nodes of every block");
    }
    for (const Block& b : mb) if (!b.vertex) throw Failure(SDG_ERR_INVALID_ARGUMENT, "null element array");
    Adjacency adj;
    try { adj = buildAdjacency(*mesh, mb); } catch (const std::runtime_error& e) { throw Failure(SDG_ERR_MESH, e.what()); }

    const double* nodes = mesh->node_coordinate;
    double extent = 0.0;
    for (int64_t i = 0; i < mesh->node_count * 3; ++i) extent = std::max(extent, std::fabs(nodes[i]));
    const double tol = 1e-12 * std::max(1.0, extent);
    size_t stateOff = 0, pointOff = 0;
    int64_t faceSlots = 0, relParts = 0;
    std::vector<CurvedMap> blockMap(mb.size());  // the order-q map of each curved block
    for (const Block& b : mb) {
      DevBlock B;
      CurvedMap& curved = blockMap[size_t(&b - mb.data())];
      B.type = b.type; B.dim = typeDim(b.type); B.p = h->p; B.ne = b.count; B.nface = typeFaces(b.type);
      B.kind = (b.type == SDG_ELEMENT_TRIANGLE || b.type == SDG_ELEMENT_TETRAHEDRON ||
                (b.type == SDG_ELEMENT_QUADRANGLE && h->p == 1))
                   ? kDense
                   : kTensor;
      B.n = h->p + 1;
      B.nb = modalCount(b.type, h->p);
      const PointRule vr = volumeRule(b.type, h->p);
      B.nq = vr.n; B.qweight = vr.w;
      B.nfq = faceRule(b.type, h->p).n;
      B.affine = 1;
      for (int64_t e = 0; e < b.count && B.affine; ++e)
        if (!isAffine(b.type, nodes, b.vertex + e * typeVertices(b.type), tol)) B.affine = 0;
      // curved elements: some geometry node off the straight (first-order) map of its element's vertices
      const int ngeo = b.geometry ? gmshNodeCount(b.type, b.geometryOrder) : 0;
      if (b.geometry) {
        curved.init(b.type, b.geometryOrder);
        const int nvt = typeVertices(b.type);
        for (int64_t e = 0; e < b.count && !B.curved; ++e) {
          const int32_t* g = b.geometry + e * ngeo;
          for (int k = 0; k < nvt; ++k)
            if (g[k] != b.vertex[e * nvt + k]) throw Failure(SDG_ERR_MESH, "geometry nodes must start with the element's vertices");
          for (int n = nvt; n < ngeo && !B.curved; ++n) {
            double X[3], J[3][3], x[3];
            gmshLatticePoint(b.type, b.geometryOrder, curved.lattice[n], X);
            jacobianAt(b.type, B.dim, nodes, b.vertex + e * nvt, X, J, x);
            for (int d = 0; d < 3; ++d)
              if (std::fabs(x[d] - nodes[size_t(g[n]) * 3 + d]) > tol) B.curved = 1;
          }
        }
      }
      if (B.curved) { B.affine = 0; h->curved = true; }
      // per-point face metrics: curved blocks, and hexahedra that are not parallelepipeds (their faces are
      // bilinear: in general neither planar nor of constant |J_f|)
      B.facePoint = B.curved || (b.type == SDG_ELEMENT_HEXAHEDRON && !B.affine);
      if (B.facePoint) h->facePoint = true;
      // geometry: affine [e][d*d+1]; bilinear tensor quads per point [e][q][d*d+1]; bilinear dense quads
      // [e][q][d*d+1] followed by the element's modal M^-1 [nb][nb] (Geometry.cpp:88-100)
      const int gs = B.dim * B.dim + 1;
      const bool denseBilinear = B.kind == kDense && !B.affine;
      B.geomStride = B.affine ? gs : (denseBilinear ? B.nq * gs + B.nb * B.nb : B.nq * gs);
      B.geomHost.assign(size_t(B.ne) * B.geomStride, 0.0);
      B.qcoord.assign(size_t(B.ne) * B.nq * 3, 0.0);
      B.minEdge.assign(size_t(B.ne), 0.0);
      std::vector<double> mphi;
      if (denseBilinear) {
        mphi.assign(size_t(B.nq) * B.nb, 0.0);
        std::vector<double> gg(size_t(B.nb) * 3);
        for (int q = 0; q < B.nq; ++q) modalBasis(b.type, h->p, &vr.x[q * 3], &mphi[size_t(q) * B.nb], gg.data());
      }
      bool bad = false;
#pragma omp parallel for schedule(static)
      for (int64_t e = 0; e < B.ne; ++e) {
        const int32_t* vv = b.vertex + e * typeVertices(b.type);
        std::vector<double> jw(B.nq);
        for (int q = 0; q < B.nq; ++q) {
          double J[3][3], x[3], A[3][3];
          if (B.curved) curved.eval(nodes, b.geometry + e * ngeo, &vr.x[q * 3], J, x);
          else jacobianAt(b.type, B.dim, nodes, vv, &vr.x[q * 3], J, x);
          for (int l = 0; l < 3; ++l) B.qcoord[(size_t(e) * B.nq + q) * 3 + l] = x[l];
          const double det = adjugate(B.dim, J, A);
          if (!(det > 0)) bad = true;
          jw[q] = det * vr.w[q];
          if (!B.affine || q == 0) {
            double* g = &B.geomHost[size_t(e) * B.geomStride + (B.affine ? 0 : size_t(q) * gs)];
            for (int r = 0; r < B.dim; ++r)
              for (int cc = 0; cc < B.dim; ++cc) g[r * B.dim + cc] = A[r][cc];
            g[B.dim * B.dim] = 1.0 / det;
          }
        }
        if (denseBilinear) {
          std::vector<double> m(size_t(B.nb) * B.nb, 0.0), inv;
          for (int i = 0; i < B.nb; ++i)
            for (int k = 0; k < B.nb; ++k) {
              double acc = 0; for (int q = 0; q < B.nq; ++q) acc += jw[q] * mphi[size_t(q) * B.nb + i] * mphi[size_t(q) * B.nb + k];
              m[size_t(i) * B.nb + k] = acc;
            }
          invertDense(B.nb, m, inv);
          std::copy(inv.begin(), inv.end(), &B.geomHost[size_t(e) * B.geomStride + size_t(B.nq) * gs]);
        }
        B.minEdge[e] = minEdgeOf(b.type, nodes, vv);
      }
      if (bad) throw Failure(SDG_ERR_MESH, "inverted or degenerate element");
      // axis-aligned affine tensor elements (structured boxes): every off-diagonal metric term is zero up to
      // the round-off of the Jacobian sums (|off| <= 1e-13 of the element's largest term); they are set to
      // zero and the stage kernel skips those products
      B.diagMetric = B.kind == kTensor && B.affine;
      for (int64_t e = 0; e < B.ne && B.diagMetric; ++e) {
        const double* g = &B.geomHost[size_t(e) * B.geomStride];
        double big = 0.0;
        for (int r = 0; r < B.dim * B.dim; ++r) big = std::max(big, std::fabs(g[r]));
        for (int r = 0; r < B.dim; ++r)
          for (int cc = 0; cc < B.dim; ++cc)
            if (r != cc && std::fabs(g[r * B.dim + cc]) > 1e-13 * big) B.diagMetric = 0;
      }
      if (B.diagMetric)
        for (int64_t e = 0; e < B.ne; ++e)
          for (int r = 0; r < B.dim; ++r)
            for (int cc = 0; cc < B.dim; ++cc)
              if (r != cc) B.geomHost[size_t(e) * B.geomStride + r * B.dim + cc] = 0.0;
      if (B.kind == kTensor) {
        B.ops.build(B.n);
        buildTensorTables(B);
      } else {
        buildDenseTables(B.type, B.p, B.tablesHost, B.phi, B.lsq);
      }
      resolveBlock(B, h->av ? 2 : (viscous ? 1 : 0), c.viscous_flux == SDG_VISCOUS_BR2 || h->av);
      if (h->av) {
        const int nvt = typeVertices(b.type);
        B.vertHost.assign(b.vertex, b.vertex + size_t(B.ne) * nvt);
        B.innerHost.resize(size_t(B.ne));
        for (int64_t e = 0; e < B.ne; ++e) B.innerHost[e] = innerRadiusOf(b.type, nodes, b.vertex + e * nvt);
        buildAvTables(B);
      }
      B.stateOffset = stateOff; stateOff += size_t(B.ne) * B.ustride;
      B.gradOffset = h->gradCount; h->gradCount += size_t(B.ne) * h->nv * B.dim * B.nb;
      if (B.facePoint) {  // outward n|J_f| at every face point of every local face, [e][f][j][d]
        const PointRule fr = faceRule(b.type, h->p);
        B.fmetricHost.assign(size_t(B.ne) * B.nface * fr.n * B.dim, 0.0);
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < B.ne; ++e)
          for (int f = 0; f < B.nface; ++f)
            for (int j = 0; j < fr.n; ++j) {
              double X[3], J[3][3], x[3], nJ[3];
              facePointInParent(b.type, f, &fr.x[j * 3], X);
              if (B.curved) curved.eval(nodes, b.geometry + e * ngeo, X, J, x);
              else jacobianAt(b.type, B.dim, nodes, b.vertex + e * typeVertices(b.type), X, J, x);
              faceNormalScaled(b.type, f, &fr.x[j * 3], J, nJ);
              for (int k = 0; k < B.dim; ++k) B.fmetricHost[((size_t(e) * B.nface + f) * fr.n + j) * B.dim + k] = nJ[k];
            }
      } else if (!B.affine || B.kind == kDense) {  // outward n|J_f| of each local face (straight faces: constant)
        B.fmetricHost.assign(size_t(B.ne) * B.nface * B.dim, 0.0);
        const int* fl = faceVertexList(b.type);
        const int nfv = typeFaceVertices(b.type);
        for (int64_t e = 0; e < B.ne; ++e) {
          const int32_t* vv = b.vertex + e * typeVertices(b.type);
          for (int f = 0; f < B.nface; ++f) {
            const double* p0 = &nodes[size_t(vv[fl[f * nfv]]) * 3];
            const double* p1 = &nodes[size_t(vv[fl[f * nfv + 1]]) * 3];
            double* m = &B.fmetricHost[(size_t(e) * B.nface + f) * B.dim];
            if (B.dim == 3) {  // triangular face: n |J_f| = (p1 - p0) x (p2 - p0) (reference area 1/2)
              const double* p2 = &nodes[size_t(vv[fl[f * nfv + 2]]) * 3];
              const double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
              const double c[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
              m[0] = a[1] * c[2] - a[2] * c[1]; m[1] = a[2] * c[0] - a[0] * c[2]; m[2] = a[0] * c[1] - a[1] * c[0];
            } else {
              const double tx = 0.5 * (p1[0] - p0[0]), ty = 0.5 * (p1[1] - p0[1]);
              m[0] = ty; m[1] = -tx;
            }
          }
        }
      }
      B.pointOffset = pointOff; pointOff += size_t(B.ne) * B.nq;
      B.faceBase = faceSlots; faceSlots += B.ne * B.nface;
      B.relOffset = relParts; relParts += B.ne;  // room for the smallest tile (one element per CTA)
      h->elements += B.ne;
      h->dof += B.ne * B.nb * h->nv;
      h->blocks.push_back(std::move(B));
    }
    h->nfq = h->blocks[0].nfq;
    h->n1d = h->blocks[0].type == SDG_ELEMENT_TETRAHEDRON ? -h->nfq : h->p + 1;
    for (int op = 0; op < kFaceOps; ++op) h->faceV[op] = facePointVariant(op, h->dim, c.convective_flux);
    h->volumePoints = int64_t(pointOff);
    h->stateCount = stateOff;
    h->faceCount = size_t(faceSlots) * h->nv * h->nfq;
    h->relParts = relParts;

    // faces: slots, orientation, straight-face geometry from the left parent's vertices (Geometry.cpp:102-169)
    const auto slotOf = [&](const FaceSide& s) { return h->blocks[s.block].faceBase + int64_t(s.element) * h->blocks[s.block].nface + s.face; };
    // per-point face geometry: [nfq][n (3), |J_f|] from the left parent's map (Geometry.cpp:102-147 on the
    // face element's own nodes, which are the parent's face nodes), and the point coordinates
    const auto faceGeomPoint = [&](const FaceSide& s, double* g, std::vector<double>* coords) {
      const DevBlock& B = h->blocks[s.block];
      const Block& b = mb[s.block];
      const PointRule fr = faceRule(B.type, B.p);
      const int ngeo = b.geometry ? gmshNodeCount(b.type, b.geometryOrder) : 0;
      const int32_t* vv = b.vertex + int64_t(s.element) * typeVertices(B.type);
      for (int j = 0; j < fr.n; ++j) {
        double X[3], J[3][3], x[3], nJ[3];
        facePointInParent(B.type, s.face, &fr.x[j * 3], X);
        if (B.curved) blockMap[s.block].eval(nodes, b.geometry + int64_t(s.element) * ngeo, X, J, x);
        else jacobianAt(B.type, B.dim, nodes, vv, X, J, x);
        faceNormalScaled(B.type, s.face, &fr.x[j * 3], J, nJ);
        const double area = std::sqrt(nJ[0] * nJ[0] + nJ[1] * nJ[1] + nJ[2] * nJ[2]);
        double* gj = g + size_t(j) * 4;
        gj[0] = nJ[0] / area; gj[1] = nJ[1] / area; gj[2] = nJ[2] / area; gj[3] = area;
        if (coords) coords->insert(coords->end(), {x[0], x[1], x[2]});
      }
    };
    const auto faceGeom = [&](const FaceSide& s, double* g, std::vector<double>* coords) {
      if (h->facePoint) { faceGeomPoint(s, g, coords); return; }
      const DevBlock& B = h->blocks[s.block];
      const int nfv = typeFaceVertices(B.type);
      const int32_t* vv = mb[s.block].vertex + int64_t(s.element) * typeVertices(B.type);
      const int* fl = faceVertexList(B.type);
      double q[4][3];
      for (int k = 0; k < nfv; ++k)
        for (int d = 0; d < 3; ++d) q[k][d] = nodes[size_t(vv[fl[s.face * nfv + k]]) * 3 + d];
      double n[3] = {0, 0, 0}, area = 0;
      if (h->dim == 1) {  // Geometry.cpp:102-112: -1 at local face 0, +1 at local face 1; measure 1
        n[0] = s.face == 0 ? -1.0 : 1.0;
        area = 1.0;
      } else if (h->dim == 2) {
        const double tx = 0.5 * (q[1][0] - q[0][0]), ty = 0.5 * (q[1][1] - q[0][1]);
        area = std::sqrt(tx * tx + ty * ty);
        n[0] = ty / area; n[1] = -tx / area;
      } else if (nfv == 3) {  // triangular face: |J_f| = |(q1 - q0) x (q2 - q0)| (reference area 1/2)
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) { a[d] = q[1][d] - q[0][d]; b[d] = q[2][d] - q[0][d]; }
        const double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        area = std::sqrt(cx * cx + cy * cy + cz * cz);
        n[0] = cx / area; n[1] = cy / area; n[2] = cz / area;
      } else {
        double planar = 0;
        for (int d = 0; d < 3; ++d) planar = std::max(planar, std::fabs(q[0][d] + q[2][d] - q[1][d] - q[3][d]));
        if (planar > tol) throw Failure(SDG_ERR_UNSUPPORTED, "non-parallelogram hexahedron face");
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) { a[d] = 0.5 * (q[1][d] - q[0][d]); b[d] = 0.5 * (q[3][d] - q[0][d]); }
        const double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        area = std::sqrt(cx * cx + cy * cy + cz * cz);
        n[0] = cx / area; n[1] = cy / area; n[2] = cz / area;
      }
      g[0] = n[0]; g[1] = n[1]; g[2] = n[2]; g[3] = area;
      if (coords) {
        const PointRule fr = faceRule(B.type, B.p);
        for (int j = 0; j < fr.n; ++j) {
          double sh[4];
          const double x = fr.x[j * 3], y = fr.x[j * 3 + 1];
          if (nfv == 1) sh[0] = 1.0;
          else if (nfv == 2) { sh[0] = 0.5 * (1 - x); sh[1] = 0.5 * (1 + x); }
          else if (nfv == 3) { sh[0] = 1 - x - y; sh[1] = x; sh[2] = y; }
          else { sh[0] = 0.25 * (1 - x) * (1 - y); sh[1] = 0.25 * (1 + x) * (1 - y); sh[2] = 0.25 * (1 + x) * (1 + y); sh[3] = 0.25 * (1 - x) * (1 + y); }
          for (int d = 0; d < 3; ++d) {
            double s = 0; for (int k = 0; k < nfv; ++k) s += sh[k] * q[k][d];
            coords->push_back(s);
          }
        }
      }
    };
    h->nInterior = int64_t(adj.interior.size());
    h->nBoundary = int64_t(adj.boundary.size());
    const int fgs = h->facePoint ? 4 * h->nfq : 4;  // face geometry doubles per face (or per face point)
    std::vector<int> fconn(size_t(h->nInterior) * 3);
    std::vector<double> fgeo(size_t(h->nInterior) * fgs);
    for (int64_t i = 0; i < h->nInterior; ++i) {
      const InteriorFace& f = adj.interior[i];
      fconn[i * 3] = int(slotOf(f.left)); fconn[i * 3 + 1] = int(slotOf(f.right)); fconn[i * 3 + 2] = f.rotation;
      faceGeom(f.left, &fgeo[i * fgs], nullptr);
    }
    std::vector<int> bconn(size_t(h->nBoundary) * 3);
    std::vector<double> bgeo(size_t(h->nBoundary) * fgs);
    for (int64_t i = 0; i < h->nBoundary; ++i) {
      const BoundaryFace& f = adj.boundary[i];
      bconn[i * 3] = int(slotOf(f.left)); bconn[i * 3 + 1] = f.condition; bconn[i * 3 + 2] = 0;
      faceGeom(f.left, &bgeo[i * fgs], &h->bcoord);
      h->bphys.push_back(f.physical);
      h->boundaryParent.push_back(f.left.block);
      h->boundaryParent.push_back(f.left.element);
      h->boundaryParent.push_back(f.left.face);
    }
    // canonical adjacency tuples
    {
      std::vector<std::array<int32_t, 7>> t;
      for (const InteriorFace& f : adj.interior)
        t.push_back({h->blocks[f.left.block].type, f.left.element, f.left.face, h->blocks[f.right.block].type,
                     f.right.element, f.right.face, f.rotation});
      std::sort(t.begin(), t.end());
      for (auto& r : t) h->adjInterior.insert(h->adjInterior.end(), r.begin(), r.end());
      std::vector<std::array<int32_t, 5>> bt;
      for (const BoundaryFace& f : adj.boundary)
        bt.push_back({h->blocks[f.left.block].type, f.left.element, f.left.face, f.physical, f.condition});
      std::sort(bt.begin(), bt.end());
      for (auto& r : bt) h->adjBoundary.insert(h->adjBoundary.end(), r.begin(), r.end());
    }

    if (device < 0) {  // host-only handle: adjacency, geometry and coordinates, no GPU
      *out = H.release();
      return SDG_OK;
    }
    SDG_CUDA(cudaSetDevice(device));
    h->hostOnly = false;
    SDG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (DevBlock& B : h->blocks) {
      for (const KernelVariant* v : {&B.stageV[0], &B.stageV[1], &B.stageV[2], &B.gradV}) {
        configureKernel(v->single, device);
        configureKernel(v->batch, device);
      }
    }
    for (const KernelVariant& v : h->faceV) { configureKernel(v.single, device); configureKernel(v.batch, device); }
    // device buffers
    h->state[0] = devAlloc<double>(h->stateCount);
    h->state[1] = devAlloc<double>(h->stateCount);
    SDG_CUDA(cudaMemsetAsync(h->state[0], 0, h->stateCount * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(h->state[1], 0, h->stateCount * 8, h->stream));
    h->face = devAlloc<double>(h->faceCount);
    SDG_CUDA(cudaMemsetAsync(h->face, 0, h->faceCount * 8, h->stream));
    if (viscousPath(h)) {
      h->faceOther = devAlloc<double>(h->faceCount);
      h->faceGrad = devAlloc<double>(h->faceCount * h->dim);
      h->faceFlux = devAlloc<double>(h->faceCount);
      h->grad = devAlloc<double>(h->gradCount);
      SDG_CUDA(cudaMemsetAsync(h->faceOther, 0, h->faceCount * 8, h->stream));
      SDG_CUDA(cudaMemsetAsync(h->faceGrad, 0, h->faceCount * h->dim * 8, h->stream));
      SDG_CUDA(cudaMemsetAsync(h->faceFlux, 0, h->faceCount * 8, h->stream));
      SDG_CUDA(cudaMemsetAsync(h->grad, 0, h->gradCount * 8, h->stream));
    }
    h->fconn = devAlloc<int>(fconn.size()); upload(h->fconn, fconn, h->stream);
    if (h->n1d < 0) {
      const std::vector<int> perm = triangleFacePermutation(h->blocks[0].type, h->p);
      h->facePerm = devAlloc<int>(perm.size()); upload(h->facePerm, perm, h->stream);
    }
    h->fgeo = devAlloc<double>(fgeo.size()); upload(h->fgeo, fgeo, h->stream);
    h->bconn = devAlloc<int>(bconn.size()); upload(h->bconn, bconn, h->stream);
    h->bgeo = devAlloc<double>(bgeo.size()); upload(h->bgeo, bgeo, h->stream);
    const size_t ghostCount = size_t(h->nBoundary) * h->nfq * (h->dim + 3);
    h->ghost = devAlloc<double>(ghostCount);
    SDG_CUDA(cudaMemsetAsync(h->ghost, 0, std::max<size_t>(ghostCount, 1) * 8, h->stream));
    h->scratch = devAlloc<double>(size_t(h->volumePoints) * h->nv);
    h->relPart = devAlloc<double>(size_t(h->relParts) * h->nv);
    h->relOut = devAlloc<double>(8);
    h->dtParts = (h->volumePoints + 255) / 256;
    h->dtPart = devAlloc<double>(size_t(h->dtParts) + 1);
    h->status = devAlloc<unsigned>(1);
    SDG_CUDA(cudaMemsetAsync(h->status, 0, sizeof(unsigned), h->stream));
    for (DevBlock& B : h->blocks) {
      B.geom = devAlloc<double>(B.geomHost.size()); upload(B.geom, B.geomHost, h->stream);
      B.tables = devAlloc<double>(B.tablesHost.size()); upload(B.tables, B.tablesHost, h->stream);
      B.minedge = devAlloc<double>(B.minEdge.size()); upload(B.minedge, B.minEdge, h->stream);
      if (!B.fmetricHost.empty()) { B.fmetric = devAlloc<double>(B.fmetricHost.size()); upload(B.fmetric, B.fmetricHost, h->stream); }
      if (B.kind == kDense) {
        B.phiDev = devAlloc<double>(B.phi.size()); upload(B.phiDev, B.phi, h->stream);
        B.lsqDev = devAlloc<double>(B.lsq.size()); upload(B.lsqDev, B.lsq, h->stream);
      }
      if (h->av) {
        B.vertDev = devAlloc<int32_t>(B.vertHost.size()); upload(B.vertDev, B.vertHost, h->stream);
        B.innerDev = devAlloc<double>(B.innerHost.size()); upload(B.innerDev, B.innerHost, h->stream);
        B.avTab = devAlloc<double>(B.avTabHost.size()); upload(B.avTab, B.avTabHost, h->stream);
        B.epsV = devAlloc<double>(B.vertHost.size());
        SDG_CUDA(cudaMemsetAsync(B.epsV, 0, B.vertHost.size() * 8, h->stream));
      }
    }
    if (h->av) {
      h->nodeAV = devAlloc<double>(size_t(h->nodeCount));
      SDG_CUDA(cudaMemsetAsync(h->nodeAV, 0, size_t(h->nodeCount) * 8, h->stream));
    }
    SDG_CUDA(cudaStreamSynchronize(h->stream));
  } catch (const Failure& f) {
    g_create_error = f.what();
    sdg_destroy(H.release());
    return f.code;
  } catch (const std::exception& ex) {
    g_create_error = ex.what();
    sdg_destroy(H.release());
    return SDG_ERR_INVALID_ARGUMENT;
  }
  *out = H.release();
  return SDG_OK;
}

int sdg_destroy(sdg_handle* h) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { delete h; return SDG_OK; }
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  dropTimingEvents(h);
  dropGraph(h);
  destroyAdjoint(h);
  for (DevBlock& B : h->blocks) {
    cudaFree(B.geom); cudaFree(B.tables); cudaFree(B.minedge); cudaFree(B.phiDev); cudaFree(B.lsqDev); cudaFree(B.fmetric);
    cudaFree(B.vertDev); cudaFree(B.innerDev); cudaFree(B.epsV); cudaFree(B.avTab);
  }
  cudaFree(h->nodeAV);
  cudaFree(h->state[0]); cudaFree(h->state[1]); cudaFree(h->face); cudaFree(h->fconn); cudaFree(h->fgeo);
  cudaFree(h->facePerm);
  cudaFree(h->bconn); cudaFree(h->bgeo); cudaFree(h->ghost); cudaFree(h->scratch); cudaFree(h->relPart);
  cudaFree(h->relOut); cudaFree(h->dtPart); cudaFree(h->status);
  cudaFree(h->faceOther); cudaFree(h->faceGrad); cudaFree(h->faceFlux); cudaFree(h->grad);
  if (h->copyStream) { cudaStreamSynchronize(h->copyStream); cudaStreamDestroy(h->copyStream); }
  if (h->copyDone) cudaEventDestroy(h->copyDone);
  if (h->stageFree) cudaEventDestroy(h->stageFree);
  cudaFree(h->inStage);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return SDG_OK;
}

int sdg_get_counts(const sdg_handle* h, sdg_counts* c) {
  if (!h || !c) return SDG_ERR_INVALID_ARGUMENT;
  std::memset(c, 0, sizeof(*c));
  c->dimension = h->dim; c->conserved_variable_count = h->nv; c->block_count = int32_t(h->blocks.size());
  for (size_t i = 0; i < h->blocks.size() && i < 2; ++i) {
    c->block_element_type[i] = h->blocks[i].type; c->block_element_count[i] = h->blocks[i].ne;
    c->block_basis_count[i] = h->blocks[i].nb; c->block_volume_point_count[i] = h->blocks[i].nq;
  }
  c->element_count = h->elements; c->volume_point_count = h->volumePoints; c->degree_of_freedom_count = h->dof;
  c->interior_face_count = h->nInterior; c->boundary_face_count = h->nBoundary; c->face_point_count = h->nfq;
  c->boundary_point_count = h->nBoundary * h->nfq;
  return SDG_OK;
}

int sdg_volume_point_coordinate(sdg_handle* h, double* out) {
  if (!h || !out) return SDG_ERR_INVALID_ARGUMENT;
  size_t off = 0;
  for (const DevBlock& B : h->blocks) { std::copy(B.qcoord.begin(), B.qcoord.end(), out + off); off += B.qcoord.size(); }
  return SDG_OK;
}

int sdg_boundary_point_coordinate(sdg_handle* h, double* out, int32_t* physical) {
  if (!h || !out) return SDG_ERR_INVALID_ARGUMENT;
  std::copy(h->bcoord.begin(), h->bcoord.end(), out);
  if (physical) std::copy(h->bphys.begin(), h->bphys.end(), physical);
  return SDG_OK;
}

int sdg_set_state_point(sdg_handle* h, const double* conserved) {
  if (!h || !conserved) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  uploadPoints(h, conserved, 0);
  traceAll(h, 0);
  if (h->gradInput == h->state[0]) h->gradInput = nullptr;
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  h->hasState = true;
  h->stateVersion++;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_set_initial_primitive(sdg_handle* h, const double* primitive) {
  if (!h || !primitive) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaMemcpyAsync(h->scratch, primitive, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyHostToDevice, h->stream));
  const int grid = int((h->volumePoints + 255) / 256);
  primitiveToConservedKernel<<<grid, 256, 0, h->stream>>>(h->scratch, h->volumePoints, h->dim, h->ph);
  checkLaunch(h);
  pointsToState(h, 0);
  traceAll(h, 0);
  if (h->gradInput == h->state[0]) h->gradInput = nullptr;
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  h->hasState = true;
  h->stateVersion++;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_set_boundary_primitive(sdg_handle* h, const double* primitive) {
  if (!h || (!primitive && h->nBoundary > 0)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  const int nv = h->nv, d = h->dim;
  const int64_t np = h->nBoundary * h->nfq;
  std::vector<double> g(size_t(np) * (d + 3));
  for (int64_t i = 0; i < np; ++i) {
    const double* pr = primitive + i * nv;
    double* o = &g[i * (d + 3)];
    const double e = h->ph.cv * pr[d + 1];
    o[0] = pr[0];
    for (int k = 0; k < d; ++k) o[1 + k] = pr[1 + k];
    o[d + 1] = e;
    // calculateComputationalFromPrimitive (VariableConvertor.cpp:368-380): the equation of state
    o[d + 2] = h->ph.incomp ? std::fma(h->ph.c02, pr[0] - h->ph.rho0, h->ph.padd) : h->ph.gm1 * pr[0] * e;
  }
  SDG_CUDA(cudaSetDevice(h->device));
  if (np > 0) SDG_CUDA(cudaMemcpyAsync(h->ghost, g.data(), g.size() * 8, cudaMemcpyHostToDevice, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_get_state_point(sdg_handle* h, double* conserved) {
  if (!h || !conserved) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  downloadPoints(h, 0, conserved);
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  return SDG_OK;
  SDG_API_END(h)
}

// Modal coefficients <-> state.  Tensor blocks: c = (Phi1^-1 x ...) U_nodal; dense blocks are modal.
static void modalConvert(sdg_handle* h, std::vector<double>& st, double* modal, bool toModal) {
  size_t moff = 0;
  for (const DevBlock& B : h->blocks) {
    const int nv = h->nv, nb = B.nb, n = B.n;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < B.ne; ++e) {
      double* u = &st[B.stateOffset + size_t(e) * B.ustride];
      double* m = modal + moff + size_t(e) * nv * nb;  // column-major (nv x nb): index b*nv + v
      if (B.kind == kDense) {
        for (int b = 0; b < nb; ++b)
          for (int v = 0; v < nv; ++v) {
            if (toModal) m[b * nv + v] = u[v * nb + b]; else u[v * nb + b] = m[b * nv + v];
          }
        continue;
      }
      std::vector<double> a(nb), t(nb);
      for (int v = 0; v < nv; ++v) {
        for (int b = 0; b < nb; ++b) a[b] = toModal ? u[v * nb + b] : m[b * nv + v];
        const double(*M)[kMaxN] = toModal ? B.ops.phi1inv : B.ops.phi1;
        // apply M along each axis: out[.., i, ..] = sum_k M[i][k] in[.., k, ..]
        const int strides[3] = {B.dim == 1 ? 1 : (B.dim == 2 ? n : n * n), B.dim == 2 ? 1 : n, 1};
        for (int ax = 0; ax < B.dim; ++ax) {
          const int st2 = strides[ax];
          for (int b = 0; b < nb; ++b) {
            const int ib = (b / st2) % n;
            const int base = b - ib * st2;
            double s = 0; for (int k = 0; k < n; ++k) s += M[ib][k] * a[base + k * st2];
            t[b] = s;
          }
          std::swap(a, t);
        }
        for (int b = 0; b < nb; ++b) { if (toModal) m[b * nv + v] = a[b]; else u[v * nb + b] = a[b]; }
      }
    }
    moff += size_t(B.ne) * nv * nb;
  }
}

int sdg_get_state_modal(sdg_handle* h, double* coefficient) {
  if (!h || !coefficient) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  std::vector<double> st(h->stateCount);
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaMemcpyAsync(st.data(), h->state[0], h->stateCount * 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  modalConvert(h, st, coefficient, true);
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_set_state_modal(sdg_handle* h, const double* coefficient) {
  if (!h || !coefficient) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  std::vector<double> st(h->stateCount, 0.0);
  modalConvert(h, st, const_cast<double*>(coefficient), false);
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaMemcpyAsync(h->state[0], st.data(), h->stateCount * 8, cudaMemcpyHostToDevice, h->stream));
  traceAll(h, 0);
  if (h->gradInput == h->state[0]) h->gradInput = nullptr;
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  h->hasState = true;
  h->stateVersion++;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_calculate_delta_time(sdg_handle* h, double cfl, double* dt) {
  if (!h || !dt || !(cfl > 0)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  if (!h->hasState) { h->err = "no state"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  stateToPoints(h, 0);
  std::vector<double> parts;
  double best = 1.79769313486231570e308;
  for (const DevBlock& B : h->blocks) {
    const int64_t np = B.ne * B.nq;
    const int grid = int((np + 255) / 256);
    deltaTimeKernel<<<grid, 256, 0, h->stream>>>(h->scratch + B.pointOffset * h->nv, B.minedge, np, B.nq, h->dim, cfl,
                                                 double(h->p + 1) * double(h->p + 1), h->ph, h->dtPart);
    checkLaunch(h);
    parts.resize(grid);
    SDG_CUDA(cudaMemcpyAsync(parts.data(), h->dtPart, grid * 8, cudaMemcpyDeviceToHost, h->stream));
    SDG_CUDA(cudaStreamSynchronize(h->stream));
    for (double x : parts) best = std::min(best, x);
  }
  *dt = best;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_step_async(sdg_handle* h, int32_t steps, double dt) {
  if (!h || steps < 0 || !std::isfinite(dt)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  if (!h->hasState) { h->err = "step before an initial state"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  for (int s = 0; s < steps; ++s) stepOnce(h, dt);  // relative error every step, as stepSolver does
  h->stateVersion++;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_step(sdg_handle* h, int32_t steps, double dt) {
  const int rc = sdg_step_async(h, steps, dt);
  if (rc != SDG_OK) return rc;
  SDG_API_BEGIN
  if (steps > 0)
    SDG_CUDA(cudaMemcpyAsync(h->relerr, h->relOut, h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  checkStatus(h);
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_step_state_point(sdg_handle* h, double dt, double* conserved, double* relative_error) {
  if (!h || !conserved || !std::isfinite(dt)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  if (!h->hasState) { h->err = "step before an initial state"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  h->pointsOut = const_cast<double*>(mappedHost(conserved));
  try {
    stepOnce(h, dt);
  } catch (...) {
    h->pointsOut = nullptr;
    throw;
  }
  h->pointsOut = nullptr;
  h->stateVersion++;
  downloadPoints(h, 0, conserved, true);
  SDG_CUDA(cudaMemcpyAsync(h->relerr, h->relOut, h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  checkStatus(h);
  if (relative_error)
    for (int v = 0; v < h->nv; ++v) relative_error[v] = h->relerr[v];
  return SDG_OK;
  SDG_API_END(h)
}

namespace {

// One step from a host state to a host state.  The input crosses the CPU-GPU link into the staging buffer on
// a stream of its own (high priority), once the previous call's conversion has consumed that buffer: the
// transfer of a call runs while the previous call's step computes.  A pinned input is read by a copy kernel
// (zero-copy), a pageable one by the copy engine.  The conversion, the traces and the step run on the handle's
// stream; the last stage of tensor blocks writes the new state into a pinned output buffer.
void stepFromTo(sdg_handle* h, double dt, const double* in, double* out) {
  const int64_t n = h->volumePoints * h->nv;
  bool allTensor = true;
  for (const DevBlock& B : h->blocks) allTensor = allTensor && B.kind == kTensor;
  if (!h->inStage) {
    const size_t stage = std::max<size_t>(size_t(n), h->stateCount);
    h->inStage = devAlloc<double>(stage);
    SDG_CUDA(cudaMemsetAsync(h->inStage, 0, stage * 8, h->stream));  // the state layout's padding stays zero
    int lo = 0, hi = 0;
    SDG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    SDG_CUDA(cudaStreamCreateWithPriority(&h->copyStream, cudaStreamNonBlocking, hi));
    SDG_CUDA(cudaEventCreateWithFlags(&h->copyDone, cudaEventDisableTiming));
    SDG_CUDA(cudaEventCreateWithFlags(&h->stageFree, cudaEventDisableTiming));
    SDG_CUDA(cudaEventRecord(h->stageFree, h->stream));
  }
  SDG_CUDA(cudaStreamWaitEvent(h->copyStream, h->stageFree, 0));
  const double* mapped = mappedHost(in);
  const int sms = multiprocessorCount(h->device);
  if (mapped && allTensor) {  // straight into the state layout: the conversion rides on the transfer
    for (const DevBlock& B : h->blocks) {
      hostCopyTensorKernel<<<unsigned(sms), 128, 0, h->copyStream>>>(
          mapped + B.pointOffset * h->nv, h->inStage + B.stateOffset, B.ne, B.nb, h->nv, B.ustride);
      SDG_CUDA(cudaGetLastError());
      h->launches++;
    }
  } else if (mapped) {
    hostCopyKernel<<<unsigned(sms), 128, 0, h->copyStream>>>(mapped, h->inStage, n);
    SDG_CUDA(cudaGetLastError());
    h->launches++;
  } else {
    SDG_CUDA(cudaMemcpyAsync(h->inStage, in, size_t(n) * 8, cudaMemcpyHostToDevice, h->copyStream));
  }
  SDG_CUDA(cudaEventRecord(h->copyDone, h->copyStream));
  SDG_CUDA(cudaStreamWaitEvent(h->stream, h->copyDone, 0));
  if (mapped && allTensor)
    SDG_CUDA(cudaMemcpyAsync(h->state[0], h->inStage, h->stateCount * 8, cudaMemcpyDeviceToDevice, h->stream));
  else
    pointsToState(h, 0, h->inStage);
  SDG_CUDA(cudaEventRecord(h->stageFree, h->stream));
  traceAll(h, 0);
  h->hasState = true;
  h->pointsOut = const_cast<double*>(mappedHost(out));
  try {
    stepOnce(h, dt);
  } catch (...) {
    h->pointsOut = nullptr;
    throw;
  }
  h->pointsOut = nullptr;
  h->stateVersion++;
  downloadPoints(h, 0, out, true);
}

}  // namespace

int sdg_step_state_point_from_async(sdg_handle* h, double dt, const double* in, double* out) {
  if (!h || !in || !out || !std::isfinite(dt)) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  stepFromTo(h, dt, in, out);
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_step_state_point_from(sdg_handle* h, double dt, const double* in, double* out, double* relative_error) {
  const int rc = sdg_step_state_point_from_async(h, dt, in, out);
  if (rc != SDG_OK) return rc;
  SDG_API_BEGIN
  SDG_CUDA(cudaMemcpyAsync(h->relerr, h->relOut, h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  checkStatus(h);
  if (relative_error)
    for (int v = 0; v < h->nv; ++v) relative_error[v] = h->relerr[v];
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_relative_error(sdg_handle* h, double* out) {
  if (!h || !out) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaMemcpyAsync(h->relerr, h->relOut, h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  for (int v = 0; v < h->nv; ++v) out[v] = h->relerr[v];
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_residual_point(sdg_handle* h, double* rate) {
  if (!h || !rate) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  if (!h->hasState) { h->err = "no state"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  // the face buffer holds the traces of state[0]: compute fluxes, then the rate without an update,
  // then restore the traces (the flux pass overwrote them)
  std::vector<Rec> recs;
  if (h->av) emitArtificialViscosity(h, -3, recs);  // the state's own artificial viscosity
  emitFluxes(h, 0, 0, recs);
  for (DevBlock& B : h->blocks) {
    Rec r = stageRec(h, B);
    r.sa.uin = h->state[0] + B.stateOffset;
    r.sa.rate = h->scratch + B.pointOffset * h->nv;
    r.sa.doVolume = 1; r.sa.doUpdate = 0; r.sa.doTrace = 0;
    recs.push_back(r);
  }
  runRecs(h, recs, h->stream);
  h->gradInput = h->state[0];
  SDG_CUDA(cudaMemcpyAsync(rate, h->scratch, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  traceAll(h, 0);
  checkStatus(h);
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_synchronize(sdg_handle* h) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  checkStatus(h);
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_launch_count(const sdg_handle* h, int64_t* n) {
  if (!h || !n) return SDG_ERR_INVALID_ARGUMENT;
  *n = h->launches;
  return SDG_OK;
}

int sdg_get_stream(const sdg_handle* h, void** stream) {
  if (!h || !stream) return SDG_ERR_INVALID_ARGUMENT;
  *stream = h->stream;
  return SDG_OK;
}

int sdg_set_kernel_timing(sdg_handle* h, int32_t enable) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  dropTimingEvents(h);
  dropGraph(h);
  h->timing = enable != 0;
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_kernel_time(sdg_handle* h, double* ms, int64_t* launches) {
  if (!h || !ms || !launches) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  SDG_API_BEGIN
  SDG_CUDA(cudaSetDevice(h->device));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  for (int k = 0; k < 5; ++k) { ms[k] = 0.0; launches[k] = 0; }
  for (size_t i = 0; i < h->timedEvents.size(); ++i) {
    float t = 0.f;
    SDG_CUDA(cudaEventElapsedTime(&t, h->timedEvents[i][0], h->timedEvents[i][1]));
    ms[h->timedClass[i]] += t;
    launches[h->timedClass[i]] += 1;
  }
  return SDG_OK;
  SDG_API_END(h)
}

int sdg_measure_fp64_peak(int32_t device, double milliseconds, double* gflops) {
  if (!gflops || !(milliseconds > 0)) return SDG_ERR_INVALID_ARGUMENT;
  try {
    *gflops = measureFp64Peak(device, milliseconds);
  } catch (const Failure& f) {
    g_create_error = f.what();
    return f.code;
  }
  return SDG_OK;
}

int sdg_measure_dmma_peak(int32_t device, int32_t shape, double milliseconds, double* gflops) {
  if (!gflops || !(milliseconds > 0) || shape < 0 || shape > 3) return SDG_ERR_INVALID_ARGUMENT;
  try {
    *gflops = measureDmmaPeak(device, shape, milliseconds);
  } catch (const Failure& f) {
    g_create_error = f.what();
    return f.code;
  }
  return SDG_OK;
}

int sdg_probe_reciprocal(int32_t device, const double* x, double* out, int64_t n) {
  if (!x || !out || n <= 0 || n > (int64_t(1) << 30)) return SDG_ERR_INVALID_ARGUMENT;
  double* d = nullptr;
  try {
    SDG_CUDA(cudaSetDevice(device));
    SDG_CUDA(cudaMalloc(&d, size_t(n) * 16));
    SDG_CUDA(cudaMemcpy(d, x, size_t(n) * 8, cudaMemcpyHostToDevice));
    reciprocalProbeKernel<<<unsigned((n + 255) / 256), 256>>>(d, d + n, n);
    SDG_CUDA(cudaGetLastError());
    SDG_CUDA(cudaMemcpy(out, d + n, size_t(n) * 8, cudaMemcpyDeviceToHost));
    SDG_CUDA(cudaFree(d));
  } catch (const Failure& f) {
    if (d) cudaFree(d);
    g_create_error = f.what();
    return f.code;
  }
  return SDG_OK;
}

int sdg_adjacency(const sdg_handle* h, int32_t* interior, int32_t* boundary) {
  if (!h) return SDG_ERR_INVALID_ARGUMENT;
  if (interior) std::copy(h->adjInterior.begin(), h->adjInterior.end(), interior);
  if (boundary) std::copy(h->adjBoundary.begin(), h->adjBoundary.end(), boundary);
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop
