// Tangent-linear model and discrete adjoint of the GB300 DG path (sdg_jvp_*, sdg_vjp_*, sdg_adjoint_steps).
//
// The reference has no differentiation; these are the spec additions.  Both are exact derivatives of
// the discrete scheme the forward path runs (same quadrature, same fluxes, same SSP-RK stages), so
//   <lambda, JVP(dU)> = <VJP(lambda), dU>
// holds to round-off, for one residual and for whole trajectories.  Scope: compressible or incompressible
// Euler and Navier-Stokes (BR1, BR2) on every element block (tensor blocks: lines, quadrangles -- affine or
// bilinear --, hexahedra; dense blocks: triangles and first-order quadrangles, affine or bilinear), the
// Boussinesq source, with or without boundary faces; artificial viscosity returns SDG_ERR_UNSUPPORTED.  The cotangents of the point-layout API are mapped
// by the transposes of the point <-> state conversions (dense blocks: Phi^T in, P^T out, P the projection).
//
// Trajectories: the tangent runs stage by stage beside the forward state.  The adjoint stores the state
// every `checkpoint_interval` steps on a forward sweep, then per segment (last first) recomputes the
// segment's stage inputs from its checkpoint and walks them backwards:
//   stage s of the step:  U_{s+1} = c0 U^n + c1 U_s + c2 dt R(U_s)
//   reverse:              lam_s = c1 lam_{s+1} + c2 dt R'(U_s)^T lam_{s+1},   lam^n += c0 lam_{s+1}
// and dJ/dmu accumulates c2 dt <lam_{s+1}, dR/dmu(U_s)>.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "sdg_internal.hpp"
#include "sdg_kernels_adjoint.cuh"

using namespace sdg;

namespace sdg {
// out += scale * sum(part[0..n)): one CTA, deterministic order (the dJ/dmu accumulator stays on the device).
__global__ void __launch_bounds__(256) muAccumulateKernel(const double* __restrict__ part, int64_t n, double scale,
                                                          double* __restrict__ out) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += part[i];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out += scale * sh[0];
}

}  // namespace sdg

// A forward trajectory kept for a later reverse sweep (sdg_forward_steps / sdg_adjoint_recorded).
struct Trajectory {
  bool valid = false;
  uint64_t version = 0;   // the handle's state version at U_N
  int steps = 0, interval = 0, segments = 0;
  double dt = 0.0;
  bool stored = false;    // every stage input kept by the forward sweep (no segment recompute)
};

struct AdjointState {
  AdjointKernels k;                    // face kernels
  std::vector<AdjointTileKernels> bk;  // element kernels of each block
  double* dU[2] = {nullptr, nullptr};
  double* dface = nullptr;
  double* dfaceOther = nullptr;
  double* dgrad = nullptr;
  double* dfaceGrad = nullptr;
  double* dflux = nullptr;
  double* lamIn = nullptr;
  double* lamStage = nullptr;
  double* lamBase = nullptr;
  double* lamU = nullptr;
  double* lamG = nullptr;
  double* lamH = nullptr;
  double* lamTr = nullptr;
  double* lamTg = nullptr;
  double* lamUp = nullptr;
  double* muPart = nullptr;
  int64_t muTiles = 0, muFaces = 0;
  double* pts = nullptr;           // point-layout conversion buffer
  std::vector<double*> pool;       // checkpoints and stage states (grown on demand)
  double* muAcc = nullptr;         // device accumulator of dJ/dmu
  double* lamGhost = nullptr;      // with boundary faces: cotangent of each boundary point's ghost primitive
  bool ghostPending = false;       // lamGhost holds a functional's own part for the next reverse sweep
  int64_t muBoundary = 0;          // dJ/dmu partial slots of the boundary kernel (Navier-Stokes)
  Trajectory traj;
  // Navier-Stokes forward quantities of every stage input of one checkpoint segment (traces, node gradient,
  // gradient traces), kept by the segment's recompute so the reverse stages read them instead of recomputing
  // them; allocated when HBM has room, else the reverse recomputes them (forwardAt)
  double* fwdStore = nullptr;
  size_t fwdSlots = 0;
  bool fwdTried = false;
  // forward quantities the reverse kernels read (null: the handle's own buffers)
  const double* curFace = nullptr;
  const double* curGrad = nullptr;
  const double* curFaceGrad = nullptr;
};

namespace sdg {
void destroyAdjoint(sdg_handle* h) {
  AdjointState* A = h->adj;
  if (!A) return;
  for (double* p : {A->dU[0], A->dU[1], A->dface, A->dfaceOther, A->dgrad, A->dfaceGrad, A->dflux, A->lamIn,
                    A->lamStage, A->lamBase, A->lamU, A->lamG, A->lamH, A->lamTr, A->lamTg, A->lamUp, A->muPart,
                    A->pts, A->muAcc, A->lamGhost})
    cudaFree(p);
  for (double* p : A->pool) cudaFree(p);
  cudaFree(A->fwdStore);
  delete A;
  h->adj = nullptr;
}
}  // namespace sdg

namespace {

double* alloc(size_t n) {
  double* p = nullptr;
  SDG_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(double)));
  return p;
}

AdjointState* adjoint(sdg_handle* h) {
  if (h->hostOnly) throw Failure(SDG_ERR_STATE, "host-only handle (created with device < 0)");
  if (!h->hasState) throw Failure(SDG_ERR_STATE, "no state");
  if (h->adj) return h->adj;
  if (h->av) throw Failure(SDG_ERR_UNSUPPORTED, "derivatives of the artificial viscosity are not built");
  std::unique_ptr<AdjointState> A(new AdjointState());
  const bool gen = h->ph.incomp || h->ph.source;
  adjointFaceKernels(h->dim, h->cfg.convective_flux, h->ns, gen, A->k);
  if (!A->k.valid()) throw Failure(SDG_ERR_UNSUPPORTED, "no derivative kernels for this configuration");
  for (const DevBlock& B : h->blocks) {
    AdjointTileKernels t;
    if (B.kind == kTensor)
      adjointTileKernels(h->dim, B.n, h->ns, h->ns && h->cfg.viscous_flux == SDG_VISCOUS_BR2, gen, B.affine != 0, t);
    else
      adjointDenseKernels(B.type, B.p, B.affine != 0, gen, h->ns, h->cfg.viscous_flux == SDG_VISCOUS_BR2, t);
    if (!t.valid() || (h->ns && !t.vjpGradient))
      throw Failure(SDG_ERR_UNSUPPORTED, "no derivative kernels for this element block");
    A->bk.push_back(t);
  }
  SDG_CUDA(cudaSetDevice(h->device));
  for (const AdjointTileKernels& t : A->bk)
    for (const void* fn : {t.jvpStage, t.vjpVolume, t.vjpGradient, t.vjpTrace}) configureKernel(fn, h->device);
  const size_t S = h->stateCount, F = h->faceCount;
  A->dU[0] = alloc(S); A->dU[1] = alloc(S);
  A->dface = alloc(F); A->dflux = alloc(F);
  A->lamIn = alloc(S); A->lamStage = alloc(S); A->lamBase = alloc(S); A->lamU = alloc(S);
  A->lamH = alloc(F); A->lamTr = alloc(F);
  if (h->ns) {
    A->dfaceOther = alloc(F); A->dgrad = alloc(h->gradCount); A->dfaceGrad = alloc(F * h->dim);
    A->lamG = alloc(h->gradCount); A->lamTg = alloc(F * h->dim); A->lamUp = alloc(F);
  }
  for (size_t b = 0; b < h->blocks.size(); ++b) A->muTiles += (h->blocks[b].ne + A->bk[b].epb - 1) / A->bk[b].epb;
  A->muFaces = (h->nInterior * h->nfq + kFaceThreads - 1) / kFaceThreads;
  A->muBoundary = h->ns ? (h->nBoundary * h->nfq + kFaceThreads - 1) / kFaceThreads : 0;
  A->muPart = alloc(size_t(A->muTiles + A->muFaces + A->muBoundary));
  A->pts = alloc(size_t(h->volumePoints) * h->nv);
  A->muAcc = alloc(1);
  SDG_CUDA(cudaMemsetAsync(A->muAcc, 0, 8, h->stream));
  if (h->nBoundary > 0) {
    A->lamGhost = alloc(size_t(h->nBoundary) * h->nfq * h->nv);
    SDG_CUDA(cudaMemsetAsync(A->lamGhost, 0, size_t(h->nBoundary) * h->nfq * h->nv * 8, h->stream));
  }
  for (double* p : {A->dU[0], A->dU[1], A->dface, A->dflux, A->lamIn, A->lamStage, A->lamBase, A->lamU, A->lamH, A->lamTr})
    SDG_CUDA(cudaMemsetAsync(p, 0, (p == A->dface || p == A->dflux || p == A->lamH || p == A->lamTr ? F : S) * 8, h->stream));
  if (h->ns) {
    SDG_CUDA(cudaMemsetAsync(A->dfaceOther, 0, F * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->dgrad, 0, h->gradCount * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->dfaceGrad, 0, F * h->dim * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->lamG, 0, h->gradCount * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->lamTg, 0, F * h->dim * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->lamUp, 0, F * 8, h->stream));
  }
  SDG_CUDA(cudaMemsetAsync(A->muPart, 0, size_t(A->muTiles + A->muFaces + A->muBoundary) * 8, h->stream));
  h->adj = A.release();
  return h->adj;
}

// Index of block B in the handle, and its element kernels.
size_t blockIndex(const sdg_handle* h, const DevBlock& B) { return size_t(&B - h->blocks.data()); }
const AdjointTileKernels& tileKernels(const sdg_handle* h, const DevBlock& B) { return h->adj->bk[blockIndex(h, B)]; }

AdjArgs baseArgs(sdg_handle* h, const DevBlock* B, const double* U) {
  AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  const AdjointState* A = h->adj;
  const double* grad = A->curGrad ? A->curGrad : h->grad;
  if (B) {
    a.u = U + B->stateOffset; a.geom = B->geom; a.tables = B->tables; a.fmetric = B->fmetric;
    a.fmetricPoint = B->facePoint;
    a.grad = h->ns ? grad + B->gradOffset : nullptr;
    a.ne = B->ne; a.faceBase = B->faceBase;
  }
  a.face = A->curFace ? A->curFace : h->face;
  a.faceGrad = A->curFaceGrad ? A->curFaceGrad : h->faceGrad;
  a.conn = h->fconn; a.fgeo = h->fgeo; a.fgeoPoint = h->facePoint ? 1 : 0; a.status = h->status;
  a.nface = h->nInterior; a.n1d = h->n1d; a.perm = h->facePerm; a.epb = B ? tileKernels(h, *B).epb : 0;
  return a;
}

void launch(sdg_handle* h, const void* fn, int64_t grid, int threads, size_t smem, AdjArgs& a, bool withPhys) {
  if (grid <= 0) return;
  Phys ph = h->ph;
  void* p[2] = {&a, &ph};
  SDG_CUDA(cudaLaunchKernel(fn, dim3(unsigned(grid)), dim3(unsigned(threads)), p, smem, h->stream));
  SDG_CUDA(cudaGetLastError());
  h->launches++;
  (void)withPhys;
}

int64_t tiles(const sdg_handle* h, const DevBlock& B) {
  const int epb = tileKernels(h, B).epb;
  return (B.ne + epb - 1) / epb;
}
int64_t faceGrid(const sdg_handle* h) { return (h->nInterior * h->nfq + kFaceThreads - 1) / kFaceThreads; }
int64_t boundaryGrid(const sdg_handle* h) { return (h->nBoundary * h->nfq + kFaceThreads - 1) / kFaceThreads; }

// Arguments of the boundary-face derivative kernels (Euler).
AdjArgs boundaryArgs(sdg_handle* h) {
  AdjArgs a = baseArgs(h, nullptr, nullptr);
  a.conn = h->bconn; a.fgeo = h->bgeo; a.nface = h->nBoundary; a.ghost = h->ghost;
  return a;
}

// Traces of state buffer `u` into `face` (the forward stage kernel's trace-only pass).
void traces(sdg_handle* h, const double* u, double* face) {
  std::vector<Rec> recs;
  for (DevBlock& B : h->blocks) {
    Rec r = stageRec(h, B);
    r.sa.uin = u + B.stateOffset;
    r.sa.face = face;
    r.sa.doTrace = 1; r.sa.doVolume = 0; r.sa.doUpdate = 0;
    recs.push_back(r);
  }
  runRecs(h, recs, h->stream);
}

// Gradient pass (BR1 or BR2) of state `u` whose traces are in `face`: neighbour traces into `other`, node gradient
// into `grad`, gradient traces into `faceGrad` (the forward kernels; linear, so they serve tangents too).
// tangent: u, face are a tangent state and its traces; the boundary exchange (the walls' states) is then the
// linearisation at the forward traces in h->face.
void gradientOf(sdg_handle* h, const double* u, double* face, double* other, double* grad, double* faceGrad,
                bool tangent = false) {
  if (grad == h->grad) h->gradInput = nullptr;  // a pass at a state that no buffer keeps
  std::vector<Rec> recs;
  Rec x = faceRec(h, kOpExchange);
  x.fa.face = face; x.fa.other = other;
  recs.push_back(x);
  if (h->nBoundary > 0 && !tangent) {
    Rec xb = faceRec(h, kOpExchangeBoundary);
    xb.fa.face = face; xb.fa.other = other;
    recs.push_back(xb);
  }
  if (h->nBoundary > 0 && tangent) {
    runRecs(h, recs, h->stream);
    recs.clear();
    AdjArgs b = baseArgs(h, nullptr, nullptr);
    b.conn = h->bconn; b.fgeo = h->bgeo; b.nface = h->nBoundary; b.ghost = h->ghost;
    b.dface = face; b.dother = other;
    launch(h, h->adj->k.jvpExchangeBoundary, (h->nBoundary * h->nfq + kFaceThreads - 1) / kFaceThreads, kFaceThreads, 0,
           b, true);
  }
  for (DevBlock& B : h->blocks) {
    Rec r = gradRec(h, B, 0);
    if (r.kind == kRecGradDense) {  // dense blocks carry their gradient pass in the dense argument block
      r.da.u = u + B.stateOffset; r.da.face = face; r.da.faceOther = other;
      r.da.grad = grad + B.gradOffset; r.da.faceGrad = faceGrad;
    } else {
      r.ga.u = u + B.stateOffset; r.ga.face = face; r.ga.faceOther = other;
      r.ga.grad = grad + B.gradOffset; r.ga.faceGrad = faceGrad;
    }
    recs.push_back(r);
  }
  runRecs(h, recs, h->stream);
}

// Forward quantities at state `u` (= state[1]): traces in h->face; NS: h->faceOther, h->grad, h->faceGrad.
void forwardAt(sdg_handle* h, const double* u) {
  traces(h, u, h->face);
  if (h->ns) gradientOf(h, u, h->face, h->faceOther, h->grad, h->faceGrad);
}

// Tangent face fluxes into dflux from tangent traces dface (and dfaceGrad), forward traces in h->face.
void tangentFaces(sdg_handle* h, double dmu) {
  AdjointState* A = h->adj;
  AdjArgs a = baseArgs(h, nullptr, nullptr);
  a.dface = A->dface; a.dfaceGrad = A->dfaceGrad; a.dflux = A->dflux; a.dmu = dmu;
  launch(h, A->k.jvpFace, faceGrid(h), kFaceThreads, 0, a, true);
  if (h->nBoundary > 0) {
    AdjArgs b = boundaryArgs(h);
    b.dface = A->dface; b.dfaceGrad = A->dfaceGrad; b.dflux = A->dflux; b.dmu = dmu;
    launch(h, A->k.jvpBoundary, boundaryGrid(h), kFaceThreads, 0, b, true);
  }
}

// Tangent element kernels: from tangent state du (traces in dface, dflux computed), write drate and/or
// the RK tangent update dout = c0 dbase + c1 du + c2dt dR with its traces.
void tangentElements(sdg_handle* h, const double* u, const double* du, double dmu, double* drate, const double* dbase,
                     double* dout, double c0, double c1, double c2dt) {
  AdjointState* A = h->adj;
  for (DevBlock& B : h->blocks) {
    AdjArgs a = baseArgs(h, &B, u);
    a.du = du + B.stateOffset;
    a.dgrad = h->ns ? A->dgrad + B.gradOffset : nullptr;
    a.dflux = A->dflux; a.dmu = dmu;
    a.drate = drate ? drate + B.stateOffset : nullptr;
    a.dbase = dbase ? dbase + B.stateOffset : nullptr;
    a.dout = dout ? dout + B.stateOffset : nullptr;
    a.dtrace = dout ? A->dface : nullptr;
    a.c0 = c0; a.c1 = c1; a.c2dt = c2dt;
    const AdjointTileKernels& t = tileKernels(h, B);
    launch(h, t.jvpStage, tiles(h, B), t.threads, t.jvpSmem, a, true);
  }
}

// Tangent of the residual at state[1] (forward quantities computed here) in direction du.
void jvpResidual(sdg_handle* h, const double* du, double dmu, double* drate) {
  AdjointState* A = h->adj;
  forwardAt(h, h->state[1]);
  traces(h, du, A->dface);
  if (h->ns) gradientOf(h, du, A->dface, A->dfaceOther, A->dgrad, A->dfaceGrad, true);
  tangentFaces(h, dmu);
  tangentElements(h, h->state[1], du, dmu, drate, nullptr, nullptr, 0.0, 0.0, 0.0);
}

// Adjoint of the residual at state[1] (forward quantities already computed by forwardAt) for cotangent lam.
// Without RK coefficients (lamStage = lamBase = null) the result R'^T lam goes to A->lamU.  For
// Navier-Stokes, A->muAcc += muScale * mu <lam, dR/dmu> on the device.
void vjpResidual(sdg_handle* h, const double* lam, const double* lamIn, double* lamStage, double* lamBase,
                 bool accumulateAll, double c0, double c1, double c2dt, double muScale, double ghostScale) {
  AdjointState* A = h->adj;
  int64_t tileOff = 0;
  for (DevBlock& B : h->blocks) {
    const AdjointTileKernels& t = tileKernels(h, B);
    AdjArgs a = baseArgs(h, &B, h->state[1]);
    a.lam = lam + B.stateOffset; a.lamU = A->lamU + B.stateOffset;
    a.lamG = h->ns ? A->lamG + B.gradOffset : nullptr;
    a.lamH = A->lamH; a.muPart = A->muPart + tileOff;
    launch(h, t.vjpVolume, tiles(h, B), t.threads, t.volSmem, a, true);
    tileOff += tiles(h, B);
  }
  {
    AdjArgs a = baseArgs(h, nullptr, nullptr);
    a.lamH = A->lamH; a.lamTr = A->lamTr; a.lamTg = A->lamTg; a.muPart = A->muPart + A->muTiles;
    launch(h, A->k.vjpFace, faceGrid(h), kFaceThreads, 0, a, true);
  }
  if (h->nBoundary > 0) {  // boundary slots of lamTr (NS: lamTg), and the ghost cotangent (weight ghostScale)
    AdjArgs b = boundaryArgs(h);
    b.lamH = A->lamH; b.lamTr = A->lamTr; b.lamTg = A->lamTg; b.lamGhost = A->lamGhost; b.ghostScale = ghostScale;
    b.muPart = A->muPart + A->muTiles + A->muFaces;
    launch(h, A->k.vjpBoundary, boundaryGrid(h), kFaceThreads, 0, b, true);
  }
  if (h->ns) {
    for (DevBlock& B : h->blocks) {
      const AdjointTileKernels& t = tileKernels(h, B);
      AdjArgs a = baseArgs(h, &B, h->state[1]);
      a.lamG = A->lamG + B.gradOffset; a.lamTg = A->lamTg; a.lamU = A->lamU + B.stateOffset; a.lamUp = A->lamUp;
      a.lamTr = A->lamTr;  // BR2: the own traces' share
      launch(h, t.vjpGradient, tiles(h, B), t.threads, t.gradSmem, a, false);
    }
    AdjArgs a = baseArgs(h, nullptr, nullptr);
    a.lamUp = A->lamUp; a.lamTr = A->lamTr;
    launch(h, A->k.vjpExchange, faceGrid(h), kFaceThreads, 0, a, false);
    if (h->nBoundary > 0) {
      AdjArgs b = boundaryArgs(h);
      b.lamUp = A->lamUp; b.lamTr = A->lamTr; b.lamGhost = A->lamGhost; b.ghostScale = ghostScale;
      launch(h, A->k.vjpExchangeBoundary, boundaryGrid(h), kFaceThreads, 0, b, true);
    }
  }
  for (DevBlock& B : h->blocks) {
    AdjArgs a = baseArgs(h, &B, h->state[1]);
    a.lamU = A->lamU + B.stateOffset; a.lamTr = A->lamTr;
    a.lamIn = lamIn ? lamIn + B.stateOffset : nullptr;
    a.lamStage = lamStage ? lamStage + B.stateOffset : nullptr;
    a.lamBase = lamBase ? lamBase + B.stateOffset : nullptr;
    a.accumulateAll = accumulateAll;
    a.c0 = c0; a.c1 = c1; a.c2dt = c2dt;
    const AdjointTileKernels& t = tileKernels(h, B);
    launch(h, t.vjpTrace, tiles(h, B), t.threads, t.traceSmem, a, false);
  }
  if (!h->ns) return;
  muAccumulateKernel<<<1, 256, 0, h->stream>>>(A->muPart, A->muTiles + A->muFaces + A->muBoundary, muScale, A->muAcc);
  SDG_CUDA(cudaGetLastError());
  h->launches++;
}

void clearGhost(sdg_handle* h) {
  if (h->adj->lamGhost)
    SDG_CUDA(cudaMemsetAsync(h->adj->lamGhost, 0, size_t(h->nBoundary) * h->nfq * h->nv * 8, h->stream));
}

double readMu(sdg_handle* h) {
  double m = 0.0;
  SDG_CUDA(cudaMemcpyAsync(&m, h->adj->muAcc, 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
  return m;
}

void uploadPoints(sdg_handle* h, const double* host, double* st) {
  AdjointState* A = h->adj;
  SDG_CUDA(cudaMemcpyAsync(A->pts, host, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyHostToDevice, h->stream));
  pointsToStateBuffer(h, A->pts, st);
}

void downloadPoints(sdg_handle* h, const double* st, double* host) {
  AdjointState* A = h->adj;
  stateToPointsBuffer(h, st, A->pts);
  SDG_CUDA(cudaMemcpyAsync(host, A->pts, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
}

// Cotangents in the point layout: the transposed conversions (on dense blocks Phi^T in, P^T out), so that the
// point-layout VJP is the transpose of the point-layout JVP.
void uploadCotangent(sdg_handle* h, const double* host, double* st) {
  AdjointState* A = h->adj;
  SDG_CUDA(cudaMemcpyAsync(A->pts, host, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyHostToDevice, h->stream));
  cotangentPointsToState(h, A->pts, st);
}

void downloadCotangent(sdg_handle* h, const double* st, double* host) {
  AdjointState* A = h->adj;
  cotangentStateToPoints(h, st, A->pts);
  SDG_CUDA(cudaMemcpyAsync(host, A->pts, size_t(h->volumePoints) * h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
  SDG_CUDA(cudaStreamSynchronize(h->stream));
}

void copyState(sdg_handle* h, double* dst, const double* src) {
  SDG_CUDA(cudaMemcpyAsync(dst, src, h->stateCount * 8, cudaMemcpyDeviceToDevice, h->stream));
}

double* poolBuffer(sdg_handle* h, size_t i) {
  AdjointState* A = h->adj;
  while (A->pool.size() <= i) A->pool.push_back(alloc(h->stateCount));
  return A->pool[i];
}

// Forward step records split by stage (records of stage s have seq / 8 == s).
std::vector<std::vector<Rec>> stepByStage(sdg_handle* h, double dt, int stages) {
  std::vector<Rec> all;
  emitStep(h, dt, false, all);
  std::vector<std::vector<Rec>> out(stages);
  for (const Rec& r : all) out[std::min(stages - 1, r.seq / 8)].push_back(r);
  return out;
}

// Tangent-linear of `steps` steps: the forward state advances too.
void jvpSteps(sdg_handle* h, int steps, double dt, double dmu) {
  AdjointState* A = h->adj;
  const int ti = h->cfg.time_integration, S = ti + 1;
  traces(h, A->dU[0], A->dface);
  const auto stages = stepByStage(h, dt, S);
  for (int n = 0; n < steps; ++n) {
    for (int s = 0; s < S; ++s) {
      const int in = s == 0 ? 0 : 1, out = s == S - 1 ? 0 : 1;
      std::vector<Rec> flux, update;
      for (const Rec& r : stages[s]) (r.seq % 8 < 3 ? flux : update).push_back(r);
      if (h->ns) {
        runRecs(h, flux, h->stream);  // forward gradient pass and viscous face fluxes (traces stay in face)
        gradientOf(h, A->dU[in], A->dface, A->dfaceOther, A->dgrad, A->dfaceGrad, true);
        tangentFaces(h, dmu);
      } else {
        tangentFaces(h, dmu);         // reads the traces before the Euler face kernel overwrites them
        runRecs(h, flux, h->stream);
      }
      tangentElements(h, h->state[in], A->dU[in], dmu, nullptr, A->dU[0], A->dU[out], kRk[ti][s][0], kRk[ti][s][1],
                      kRk[ti][s][2] * dt);
      runRecs(h, update, h->stream);
    }
  }
  h->gradInput = stepGradientInput(h);
}

void releaseForwardStore(sdg_handle* h);

// Pool buffers [first, first + count) allocated, when the device keeps at least 2 GiB free beside the ones
// still missing; false (nothing allocated) otherwise.
bool reservePool(sdg_handle* h, size_t first, size_t count) {
  AdjointState* A = h->adj;
  const size_t have = A->pool.size() > first ? std::min(A->pool.size() - first, count) : 0;
  const size_t missing = count - have;
  size_t freeB = 0, totalB = 0;
  SDG_CUDA(cudaMemGetInfo(&freeB, &totalB));
  if (missing * h->stateCount * sizeof(double) + (size_t(2) << 30) > freeB) return false;
  for (size_t i = 0; i < count; ++i) poolBuffer(h, first + i);
  return true;
}

// Forward sweep of `steps` steps from the current state U_0, keeping U every `interval` steps
// (pool[0..segments)) and U_N (pool[segments]); records the trajectory for the reverse sweep.  With the
// trajectory store on and HBM room for all steps x stages states, every stage input is kept as well
// (pool[segments + 1 + n S + s]): the reverse sweep then reads them instead of recomputing each segment.
void forwardSweep(sdg_handle* h, int steps, double dt, int interval) {
  AdjointState* A = h->adj;
  const int segments = (steps + interval - 1) / interval;
  const int S = h->cfg.time_integration + 1;
  const size_t storeBase = size_t(segments) + 1;
  std::vector<Rec> recs;
  emitStep(h, dt, true, recs);
  bool stored = false;
  if (h->adjointTrajectoryStore) {
    releaseForwardStore(h);  // the stored trajectory replaces the per-segment forward store
    stored = reservePool(h, 0, storeBase + size_t(steps) * S);
  }
  if (stored) {
    std::vector<std::vector<Rec>> stage(S);  // the step's records by stage (the reduction with the last)
    for (const Rec& r : recs) stage[std::min(S - 1, r.seq / 8)].push_back(r);
    for (int n = 0; n < steps; ++n) {
      if (n % interval == 0) copyState(h, poolBuffer(h, n / interval), h->state[0]);
      for (int s = 0; s < S; ++s) {
        copyState(h, poolBuffer(h, storeBase + size_t(n) * S + s), h->state[s == 0 ? 0 : 1]);
        runRecs(h, stage[s], h->stream);
      }
    }
  } else {
    for (int g = 0; g < segments; ++g) {
      copyState(h, poolBuffer(h, g), h->state[0]);
      const int n = std::min(interval, steps - g * interval);
      for (int k = 0; k < n; ++k) runRecs(h, recs, h->stream);
    }
  }
  copyState(h, poolBuffer(h, segments), h->state[0]);
  h->stateVersion++;
  h->gradInput = stepGradientInput(h);
  A->traj.valid = true;
  A->traj.version = h->stateVersion;
  A->traj.steps = steps; A->traj.interval = interval; A->traj.segments = segments; A->traj.dt = dt;
  A->traj.stored = stored;
}

// Doubles of one stored stage input: traces, node gradient, gradient traces.
size_t fwdSlotSize(const sdg_handle* h) { return h->faceCount * (1 + h->dim) + h->gradCount; }

// The forward store for `slots` stage inputs, allocated once when the device keeps at least 2 GiB free
// beside it; false (recompute in the reverse) otherwise.
bool forwardStore(sdg_handle* h, size_t slots) {
  AdjointState* A = h->adj;
  if (!h->ns) return false;
  if (A->fwdStore && A->fwdSlots >= slots) return true;
  if (A->fwdTried && !A->fwdStore) return false;
  cudaFree(A->fwdStore);
  A->fwdStore = nullptr; A->fwdSlots = 0; A->fwdTried = true;
  size_t freeB = 0, totalB = 0;
  SDG_CUDA(cudaMemGetInfo(&freeB, &totalB));
  const size_t bytes = slots * fwdSlotSize(h) * sizeof(double);
  if (bytes + (size_t(2) << 30) > freeB) return false;
  if (cudaMalloc(&A->fwdStore, bytes) != cudaSuccess) {
    cudaGetLastError();
    A->fwdStore = nullptr;
    return false;
  }
  A->fwdSlots = slots;
  return true;
}

double* fwdSlot(sdg_handle* h, size_t i) { return h->adj->fwdStore + i * fwdSlotSize(h); }

void releaseForwardStore(sdg_handle* h) {
  AdjointState* A = h->adj;
  if (A->fwdStore) cudaFree(A->fwdStore);
  A->fwdStore = nullptr; A->fwdSlots = 0; A->fwdTried = false;
}

// Keep the traces of the current stage input (h->face) in stored slot i.
void keepTraces(sdg_handle* h, size_t i) {
  SDG_CUDA(cudaMemcpyAsync(fwdSlot(h, i), h->face, h->faceCount * 8, cudaMemcpyDeviceToDevice, h->stream));
}

// Records of one stage whose node gradient and gradient traces live in stored slot i: the gradient kernels
// write them there and the face and stage kernels read them there (no copy).
std::vector<Rec> intoSlot(sdg_handle* h, const std::vector<Rec>& recs, size_t i) {
  double* g = fwdSlot(h, i) + h->faceCount;
  double* fg = g + h->gradCount;
  const auto rebase = [&](auto* p, const double* from, size_t count, double* to) {
    using P = decltype(p);
    if (p && p >= from && p < from + count) return P(to + (p - from));
    return p;
  };
  std::vector<Rec> out = recs;
  const size_t G = h->gradCount, FG = h->faceCount * h->dim;
  for (Rec& r : out) {
    r.ga.grad = rebase(r.ga.grad, h->grad, G, g); r.ga.faceGrad = rebase(r.ga.faceGrad, h->faceGrad, FG, fg);
    r.da.grad = rebase(r.da.grad, h->grad, G, g); r.da.faceGrad = rebase(r.da.faceGrad, h->faceGrad, FG, fg);
    r.fa.faceGrad = rebase(r.fa.faceGrad, h->faceGrad, FG, fg);
    r.sa.grad = rebase(r.sa.grad, h->grad, G, g);
  }
  return out;
}

void useForward(sdg_handle* h, size_t i) {
  AdjointState* A = h->adj;
  const double* d = fwdSlot(h, i);
  A->curFace = d; A->curGrad = d + h->faceCount; A->curFaceGrad = d + h->faceCount + h->gradCount;
}

void useOwnForward(sdg_handle* h) {
  AdjointState* A = h->adj;
  A->curFace = A->curGrad = A->curFaceGrad = nullptr;
}

// Reverse sweep of the recorded trajectory: on entry A->lamIn holds dJ/dU_N; on exit it holds dJ/dU_0 and
// the state is U_N again.  Returns dJ/dmu (Navier-Stokes; 0 for Euler).
double backwardSweep(sdg_handle* h) {
  AdjointState* A = h->adj;
  const Trajectory T = A->traj;
  const int ti = h->cfg.time_integration, S = ti + 1;
  const int steps = T.steps, interval = T.interval, segments = T.segments;
  const double dt = T.dt;
  const size_t storeBase = size_t(segments) + 1;
  const auto stages = stepByStage(h, dt, S);
  const bool stored = T.stored;  // every stage input kept by the forward sweep: no recompute
  const bool keep = !stored && forwardStore(h, size_t(interval) * S);
  SDG_CUDA(cudaMemsetAsync(A->lamBase, 0, h->stateCount * 8, h->stream));
  SDG_CUDA(cudaMemsetAsync(A->muAcc, 0, 8, h->stream));
  if (!A->ghostPending) clearGhost(h);  // a functional's cotangent may have left its own ghost part
  A->ghostPending = false;
  const double muScale = h->ns && h->ph.mu > 0.0 ? 1.0 / h->ph.mu : 0.0;
  for (int g = segments - 1; g >= 0; --g) {
    const int n0 = g * interval, n1 = std::min(steps, n0 + interval);
    // recompute the segment from its checkpoint, keeping every stage input (and, with room, its forward
    // quantities: the flux records leave the traces, gradient and gradient traces of the stage input)
    if (!stored) {
      copyState(h, h->state[0], poolBuffer(h, g));
      traces(h, h->state[0], h->face);
      for (int n = n0; n < n1; ++n)
        for (int s = 0; s < S; ++s) {
          const size_t slot = size_t(n - n0) * S + s;
          copyState(h, poolBuffer(h, storeBase + slot), h->state[s == 0 ? 0 : 1]);
          if (keep) {
            keepTraces(h, slot);
            runRecs(h, intoSlot(h, stages[s], slot), h->stream);
          } else {
            runRecs(h, stages[s], h->stream);
          }
        }
    }
    // reverse
    for (int n = n1 - 1; n >= n0; --n)
      for (int s = S - 1; s >= 0; --s) {
        const size_t slot = stored ? size_t(n) * S + s : size_t(n - n0) * S + s;
        copyState(h, h->state[1], poolBuffer(h, storeBase + slot));
        if (keep) useForward(h, slot);
        else forwardAt(h, h->state[1]);
        const double c0 = kRk[ti][s][0], c1 = kRk[ti][s][1], c2dt = kRk[ti][s][2] * dt;
        if (s > 0) {
          vjpResidual(h, A->lamIn, A->lamIn, A->lamStage, A->lamBase, false, c0, c1, c2dt, c2dt * muScale, c2dt);
          std::swap(A->lamIn, A->lamStage);
        } else {
          vjpResidual(h, A->lamIn, A->lamIn, nullptr, A->lamBase, true, c0, c1, c2dt, c2dt * muScale, c2dt);
          std::swap(A->lamIn, A->lamBase);
          SDG_CUDA(cudaMemsetAsync(A->lamBase, 0, h->stateCount * 8, h->stream));
        }
        useOwnForward(h);
      }
  }
  copyState(h, h->state[0], poolBuffer(h, segments));
  traces(h, h->state[0], h->face);
  return h->ns ? readMu(h) : 0.0;
}

// Device inputs of the surface-force kernels for boundary group `physical` (1-based mesh physical index).
struct ForceInputs {
  int* select = nullptr;
  double* fw = nullptr;
  double* out = nullptr;
  ~ForceInputs() { cudaFree(select); cudaFree(fw); cudaFree(out); }
};

ForceArgs forceInputs(sdg_handle* h, int physical, ForceInputs& in, bool pointOut) {
  if (h->nBoundary == 0) throw Failure(SDG_ERR_INVALID_ARGUMENT, "the mesh has no boundary faces");
  std::vector<int> sel(size_t(h->nBoundary));
  bool any = false;
  for (int64_t i = 0; i < h->nBoundary; ++i) { sel[i] = h->bphys[i] == physical; any = any || sel[i]; }
  if (!any) throw Failure(SDG_ERR_INVALID_ARGUMENT, "no boundary face belongs to that physical group");
  const PointRule fr = faceRule(h->blocks[0].type, h->p);
  SDG_CUDA(cudaMalloc(&in.select, sel.size() * sizeof(int)));
  SDG_CUDA(cudaMalloc(&in.fw, fr.w.size() * 8));
  SDG_CUDA(cudaMemcpyAsync(in.select, sel.data(), sel.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  SDG_CUDA(cudaMemcpyAsync(in.fw, fr.w.data(), fr.w.size() * 8, cudaMemcpyHostToDevice, h->stream));
  if (pointOut) SDG_CUDA(cudaMalloc(&in.out, size_t(h->nBoundary) * h->nfq * h->dim * 8));
  ForceArgs a;
  std::memset(&a, 0, sizeof(a));
  a.face = h->face; a.faceGrad = h->faceGrad; a.conn = h->bconn; a.fgeo = h->bgeo; a.select = in.select;
  a.fgeoPoint = h->facePoint ? 1 : 0;
  a.fw = in.fw; a.out = in.out; a.nface = h->nBoundary; a.n1d = h->n1d; a.ns = h->ns ? 1 : 0;
  return a;
}

int adjFail(sdg_handle* h, const Failure& f) {
  h->err = f.what();
  return f.code;
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

int sdg_volume_point_weight(sdg_handle* h, double* weight) {
  if (!h || !weight) return SDG_ERR_INVALID_ARGUMENT;
  for (const DevBlock& B : h->blocks) {
    const int gs = B.dim * B.dim + 1;
    for (int64_t e = 0; e < B.ne; ++e)
      for (int q = 0; q < B.nq; ++q) {
        const double jinv = B.affine ? B.geomHost[size_t(e) * B.geomStride + gs - 1]
                                     : B.geomHost[size_t(e) * B.geomStride + size_t(q) * gs + gs - 1];
        weight[B.pointOffset + size_t(e) * B.nq + q] = B.qweight[q] / jinv;
      }
  }
  return SDG_OK;
}

int sdg_set_viscosity(sdg_handle* h, double mu) {
  if (!h || !(mu >= 0.0) || !std::isfinite(mu)) return SDG_ERR_INVALID_ARGUMENT;
  h->cfg.dynamic_viscosity = mu;
  h->ph.mu = mu;
  h->ph.kappa = h->cfg.prandtl_number > 0 ? h->cfg.specific_heat_constant_pressure * mu / h->cfg.prandtl_number : 0.0;
  dropGraph(h);
  h->stateVersion++;
  return SDG_OK;
}

int sdg_jvp_residual(sdg_handle* h, const double* tangent, double viscosity_tangent, double* rate_tangent) {
  if (!h || !tangent || !rate_tangent || !std::isfinite(viscosity_tangent)) return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    copyState(h, h->state[1], h->state[0]);
    uploadPoints(h, tangent, A->dU[0]);
    jvpResidual(h, A->dU[0], viscosity_tangent, A->dU[1]);
    downloadPoints(h, A->dU[1], rate_tangent);
    traces(h, h->state[0], h->face);
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_vjp_residual(sdg_handle* h, const double* rate_cotangent, double* cotangent, double* viscosity_cotangent) {
  if (!h || !rate_cotangent || !cotangent) return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    copyState(h, h->state[1], h->state[0]);
    uploadCotangent(h, rate_cotangent, A->lamIn);
    forwardAt(h, h->state[1]);
    SDG_CUDA(cudaMemsetAsync(A->muAcc, 0, 8, h->stream));
    clearGhost(h);
    A->ghostPending = false;
    vjpResidual(h, A->lamIn, nullptr, nullptr, nullptr, false, 0.0, 0.0, 0.0,
                h->ns && h->ph.mu > 0.0 ? 1.0 / h->ph.mu : 0.0, 1.0);
    downloadCotangent(h, A->lamU, cotangent);
    if (viscosity_cotangent) *viscosity_cotangent = h->ns ? readMu(h) : 0.0;
    traces(h, h->state[0], h->face);
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_jvp_steps(sdg_handle* h, int32_t steps, double dt, const double* tangent_in, double viscosity_tangent,
                  double* tangent_out) {
  if (!h || steps < 0 || !tangent_in || !tangent_out || !std::isfinite(dt) || !std::isfinite(viscosity_tangent))
    return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    uploadPoints(h, tangent_in, A->dU[0]);
    jvpSteps(h, steps, dt, viscosity_tangent);
    h->stateVersion++;
    downloadPoints(h, A->dU[0], tangent_out);
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_adjoint_steps(sdg_handle* h, int32_t steps, double dt, int32_t interval, const double* final_cotangent,
                      double* initial_cotangent, double* viscosity_cotangent) {
  if (!h || steps < 1 || interval < 1 || !final_cotangent || !initial_cotangent || !std::isfinite(dt))
    return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    forwardSweep(h, steps, dt, interval);
    uploadCotangent(h, final_cotangent, A->lamIn);
    const double m = backwardSweep(h);
    downloadCotangent(h, A->lamIn, initial_cotangent);
    if (viscosity_cotangent) *viscosity_cotangent = m;
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_forward_steps(sdg_handle* h, int32_t steps, double dt, int32_t interval) {
  if (!h || steps < 1 || interval < 1 || !std::isfinite(dt)) return SDG_ERR_INVALID_ARGUMENT;
  try {
    adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    forwardSweep(h, steps, dt, interval);
    SDG_CUDA(cudaMemcpyAsync(h->relerr, h->relOut, h->nv * 8, cudaMemcpyDeviceToHost, h->stream));
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_adjoint_recorded(sdg_handle* h, const double* final_cotangent, double* initial_cotangent,
                         double* viscosity_cotangent) {
  if (!h || !final_cotangent || !initial_cotangent) return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    if (!A->traj.valid || A->traj.version != h->stateVersion)
      throw Failure(SDG_ERR_STATE, "no recorded trajectory ends at the current state (sdg_forward_steps first)");
    SDG_CUDA(cudaSetDevice(h->device));
    uploadCotangent(h, final_cotangent, A->lamIn);
    const double m = backwardSweep(h);
    downloadCotangent(h, A->lamIn, initial_cotangent);
    if (viscosity_cotangent) *viscosity_cotangent = m;
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_surface_force(sdg_handle* h, int32_t physical, double* force) {
  if (!h || !force) return SDG_ERR_INVALID_ARGUMENT;
  if (h->hostOnly) { h->err = "host-only handle (created with device < 0)"; return SDG_ERR_STATE; }
  if (!h->hasState) { h->err = "no state"; return SDG_ERR_STATE; }
  try {
    SDG_CUDA(cudaSetDevice(h->device));
    // the gradient traces of the current state (the step leaves those of its last stage input)
    if (h->ns) gradientOf(h, h->state[0], h->face, h->faceOther, h->grad, h->faceGrad);
    ForceInputs in;
    const ForceArgs a = forceInputs(h, physical, in, true);
    const int64_t pts = h->nBoundary * h->nfq;
    const unsigned grid = unsigned((pts + kFaceThreads - 1) / kFaceThreads);
    if (h->dim == 1) surfaceForceKernel<1><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph);
    else if (h->dim == 2) surfaceForceKernel<2><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph);
    else surfaceForceKernel<3><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph);
    SDG_CUDA(cudaGetLastError());
    h->launches++;
    std::vector<double> part(size_t(pts) * h->dim);
    SDG_CUDA(cudaMemcpyAsync(part.data(), in.out, part.size() * 8, cudaMemcpyDeviceToHost, h->stream));
    SDG_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < h->dim; ++k) force[k] = 0.0;
    for (int64_t i = 0; i < pts; ++i)
      for (int k = 0; k < h->dim; ++k) force[k] += part[size_t(i) * h->dim + k];
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_surface_force_cotangent(sdg_handle* h, int32_t physical, const double* direction, double* cotangent) {
  if (!h || !direction || !cotangent) return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    SDG_CUDA(cudaSetDevice(h->device));
    // forward quantities of the current state: traces (kept by the step) and, NS, the gradient pass
    if (h->ns) gradientOf(h, h->state[0], h->face, h->faceOther, h->grad, h->faceGrad);
    ForceInputs in;
    ForceArgs a = forceInputs(h, physical, in, false);
    for (int k = 0; k < h->dim; ++k) a.dir[k] = direction[k];
    a.out = A->lamTr;
    SDG_CUDA(cudaMemsetAsync(A->lamTr, 0, h->faceCount * 8, h->stream));
    SDG_CUDA(cudaMemsetAsync(A->lamU, 0, h->stateCount * 8, h->stream));
    if (h->ns) {
      SDG_CUDA(cudaMemsetAsync(A->lamTg, 0, h->faceCount * h->dim * 8, h->stream));
      SDG_CUDA(cudaMemsetAsync(A->lamG, 0, h->gradCount * 8, h->stream));
    }
    clearGhost(h);
    const int64_t pts = h->nBoundary * h->nfq;
    const unsigned grid = unsigned((pts + kFaceThreads - 1) / kFaceThreads);
    if (h->dim == 1) surfaceForceTraceCotangentKernel<1><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph, A->lamTg);
    else if (h->dim == 2) surfaceForceTraceCotangentKernel<2><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph, A->lamTg);
    else surfaceForceTraceCotangentKernel<3><<<grid, kFaceThreads, 0, h->stream>>>(a, h->ph, A->lamTg);
    SDG_CUDA(cudaGetLastError());
    h->launches++;
    if (h->ns) {  // the gradient traces' cotangent back through the gradient pass (vjpResidual's NS part)
      for (DevBlock& B : h->blocks) {
        AdjArgs g = baseArgs(h, &B, h->state[0]);
        g.lamG = A->lamG + B.gradOffset; g.lamTg = A->lamTg; g.lamU = A->lamU + B.stateOffset; g.lamUp = A->lamUp;
        g.lamTr = A->lamTr;
        const AdjointTileKernels& t = tileKernels(h, B);
        launch(h, t.vjpGradient, tiles(h, B), t.threads, t.gradSmem, g, false);
      }
      AdjArgs x = baseArgs(h, nullptr, nullptr);
      x.lamUp = A->lamUp; x.lamTr = A->lamTr;
      launch(h, A->k.vjpExchange, faceGrid(h), kFaceThreads, 0, x, false);
      AdjArgs b = boundaryArgs(h);
      b.lamUp = A->lamUp; b.lamTr = A->lamTr; b.lamGhost = A->lamGhost; b.ghostScale = 1.0;
      launch(h, A->k.vjpExchangeBoundary, boundaryGrid(h), kFaceThreads, 0, b, true);
    }
    A->ghostPending = true;  // the functional's own ghost dependence joins the next reverse sweep's
    // the transposed trace operator: lamU += T^T lamTr (the element kernel of the reverse without its
    // volume and RK parts)
    for (DevBlock& B : h->blocks) {
      AdjArgs t = baseArgs(h, &B, h->state[0]);
      t.lamU = A->lamU + B.stateOffset; t.lamTr = A->lamTr;
      const AdjointTileKernels& tk = tileKernels(h, B);
      launch(h, tk.vjpTrace, tiles(h, B), tk.threads, tk.traceSmem, t, false);
    }
    downloadCotangent(h, A->lamU, cotangent);
    checkStatus(h);
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_adjoint_boundary_cotangent(sdg_handle* h, double* out) {
  if (!h || !out) return SDG_ERR_INVALID_ARGUMENT;
  try {
    AdjointState* A = adjoint(h);
    const size_t n = size_t(h->nBoundary) * h->nfq * h->nv;
    if (n == 0) return SDG_OK;
    SDG_CUDA(cudaSetDevice(h->device));
    SDG_CUDA(cudaMemcpyAsync(out, A->lamGhost, n * 8, cudaMemcpyDeviceToHost, h->stream));
    SDG_CUDA(cudaStreamSynchronize(h->stream));
  } catch (const Failure& f) {
    return adjFail(h, f);
  }
  return SDG_OK;
}

int sdg_set_adjoint_trajectory_store(sdg_handle* h, int32_t enable) {
  if (!h || (enable != 0 && enable != 1)) return SDG_ERR_INVALID_ARGUMENT;
  h->adjointTrajectoryStore = enable != 0;
  if (h->adj) h->adj->traj.valid = false;  // a recorded trajectory was kept under the other scheme
  return SDG_OK;
}

int sdg_adjoint_memory(sdg_handle* h, int64_t* bytes) {
  if (!h || !bytes) return SDG_ERR_INVALID_ARGUMENT;
  *bytes = 0;
  if (!h->adj) return SDG_OK;
  const AdjointState* A = h->adj;
  *bytes = int64_t(A->pool.size()) * int64_t(h->stateCount) * 8;
  if (A->fwdStore) *bytes += int64_t(A->fwdSlots) * int64_t(fwdSlotSize(h)) * 8;
  return SDG_OK;
}

}  // extern "C"
#pragma GCC visibility pop
