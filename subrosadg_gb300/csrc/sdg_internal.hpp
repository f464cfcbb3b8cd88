// Internal host structures of the GB300 DG library: the problem handle, its element blocks, and the
// launch records every execution mode (one instance, CUDA graph, batched persistent launches,
// autotuning) is built from.  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sdg_gpu.h"
#include "sdg_kernels_dense.cuh"
#include "sdg_kernels_ns.cuh"
#include "sdg_mesh.hpp"
#include "sdg_operators.hpp"
#include "sdg_variants.hpp"

namespace sdg {

struct Failure : std::runtime_error {
  int code;
  Failure(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define SDG_CUDA(call)                                                                              \
  do {                                                                                              \
    cudaError_t _e = (call);                                                                        \
    if (_e != cudaSuccess)                                                                          \
      throw ::sdg::Failure(_e == cudaErrorMemoryAllocation ? SDG_ERR_OUT_OF_MEMORY : SDG_ERR_CUDA,   \
                           std::string(#call) + ": " + cudaGetErrorString(_e));                     \
  } while (0)

enum Kind { kTensor = 0, kDense = 1 };

struct DevBlock {
  int type = 0, dim = 2, p = 1, n = 0, kind = kTensor, affine = 1;
  int diagMetric = 0;              // affine tensor block whose metric terms |J| dxi/dx are all diagonal
  int curved = 0;                  // block with curved (high-order) elements
  int facePoint = 0;               // face metrics per face point (curved blocks, hexahedra not parallelepipeds)
  int nb = 0, nq = 0, nface = 0, nfq = 0, ustride = 0, fstride = 0, geomStride = 0;
  int64_t ne = 0, faceBase = 0;
  size_t stateOffset = 0;          // doubles
  size_t pointOffset = 0;          // volume points before this block
  std::vector<double> qcoord;      // [e][q][3]
  std::vector<double> qweight;     // reference weights [q]
  std::vector<double> minEdge;     // [e]
  std::vector<double> geomHost;
  std::vector<double> tablesHost;
  std::vector<double> phi;         // dense: [q][nb] ; tensor: unused
  std::vector<double> lsq;         // dense: [nb][q] projection (Phi^T Phi)^-1 Phi^T, then its [nb] row sums
  TensorOps ops;
  double* geom = nullptr;
  double* tables = nullptr;
  double* minedge = nullptr;
  double* phiDev = nullptr;
  double* lsqDev = nullptr;
  KernelVariant stageV[3];         // stage kernels: [0] Euler, [1] Navier-Stokes, [2] artificial viscosity
  KernelVariant gradV;             // gradient kernel (Navier-Stokes)
  int epb = 0, threads = 0;        // stage tile: elements per CTA, threads per CTA
  int64_t grid = 0;                // stage tiles (CTAs of a one-instance launch)
  size_t smem = 0;
  int gepb = 0, gthreads = 0;      // gradient tile
  int64_t ggrid = 0;
  size_t gsmem = 0;
  std::vector<double> fmetricHost; // [e][nface][d] outward n|J_f| (bilinear and dense blocks)
  double* fmetric = nullptr;
  size_t gradOffset = 0;           // doubles into the gradient buffer
  int64_t relOffset = 0;           // first relative-error partial slot (one slot per possible tile)
  // artificial viscosity: element vertices (mesh nodes), inner radius, vertex values, tables
  std::vector<int32_t> vertHost;   // [e][nvert]
  std::vector<double> innerHost;   // [e]
  std::vector<double> avTabHost;
  int32_t* vertDev = nullptr;
  double* innerDev = nullptr;
  double* epsV = nullptr;          // [e][nvert]
  double* avTab = nullptr;
};

// One kernel launch of a step: the kernel pair, its one-instance launch shape and its arguments.
enum RecKind { kRecStage = 0, kRecGradTensor = 1, kRecGradDense = 2, kRecFace = 3, kRecRelerr = 4, kRecAv = 5 };
struct Rec {
  int kind = 0;
  int cls = 0;                     // timing class: 0 element, 1 interior face, 2 boundary face, 3 reduction, 4 gradient
  int seq = 0;                     // dependency level: records of one level are independent
  const void* fn = nullptr;        // one-instance kernel
  const void* bfn = nullptr;       // batched persistent kernel
  int threads = 0, epb = 0;
  size_t smem = 0;
  int64_t units = 0;               // CTAs of the one-instance launch (tiles / point chunks / variables)
  int soloThreads = 0;             // face records of small meshes: narrower CTAs for the one-instance launch
  int64_t soloUnits = 0;           // (the batched work lists keep threads / units)
  StageArgs sa;
  Phys ph;
  GradArgs ga;
  DenseGradArgs da;
  FaceArgs fa;
  RelArgs ra;
  AvArgs av;
};

// Sets the dynamic shared memory limit of a kernel to the device's opt-in maximum (once per device).
void configureKernel(const void* fn, int device);
int sharedMemoryOptin(int device);
int multiprocessorCount(int device);

}  // namespace sdg

struct sdg_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  sdg_config cfg{};
  sdg::Phys ph{};
  int dim = 2, nv = 4, p = 1;
  std::vector<sdg::DevBlock> blocks;
  sdg::KernelVariant faceV[sdg::kFaceOps];  // face-point kernels per FaceOp
  double* state[2] = {nullptr, nullptr};
  size_t stateCount = 0;
  double* face = nullptr;
  size_t faceCount = 0;
  bool ns = false;                 // Navier-Stokes: gradient pass + viscous fluxes
  bool av = false;                 // artificial viscosity: gradient pass + artificial viscous fluxes
  double* nodeAV = nullptr;        // artificial viscosity per mesh node [nodeCount]
  double* faceOther = nullptr;     // NS: neighbour traces
  double* faceGrad = nullptr;      // NS: gradient traces
  double* faceFlux = nullptr;      // NS: face fluxes
  double* grad = nullptr;          // NS: total gradient at the nodes
  const double* gradInput = nullptr;  // NS: state buffer the last gradient pass read, while it still holds
                                      // that input (null when not kept)
  size_t gradCount = 0;
  int* fconn = nullptr; double* fgeo = nullptr; int64_t nInterior = 0;
  int* bconn = nullptr; double* bgeo = nullptr; double* ghost = nullptr; int64_t nBoundary = 0;
  int nfq = 0, n1d = 0;           // n1d < 0: triangular faces of -n1d points, paired through facePerm
  int* facePerm = nullptr;        // [3][nfq] right point of left point j at rotation r (triangular faces)
  std::vector<int32_t> adjInterior, adjBoundary;
  std::vector<double> bcoord; std::vector<int32_t> bphys;
  std::vector<int32_t> boundaryParent;  // per boundary face: (block, element, local face) of its parent
  std::vector<int64_t> boundaryOrder;   // sdg_set_boundary_face_order: library boundary face of each caller position
  int64_t nodeCount = 0;                // mesh nodes (raw-binary files carry one value per node)
  double* scratch = nullptr;       // point-layout conversion buffer [volume_points][nv]
  // sdg_step_state_point_from: staging buffer of the input state [volume_points][nv], the stream its transfers
  // run on, and the events that order a transfer after the previous conversion and before its own (on first use)
  double* inStage = nullptr;
  cudaStream_t copyStream = nullptr;
  cudaEvent_t copyDone = nullptr, stageFree = nullptr;
  int64_t volumePoints = 0;
  double* relPart = nullptr; int64_t relParts = 0;
  double* relOut = nullptr; double* dtPart = nullptr; int64_t dtParts = 0;
  unsigned* status = nullptr;
  double relerr[5] = {0, 0, 0, 0, 0};
  bool hasState = false;
  bool hostOnly = true;            // created with device < 0: no GPU resources
  int64_t launches = 0;
  bool timing = false;             // bracket launches with events (sdg_set_kernel_timing)
  std::vector<std::array<cudaEvent_t, 2>> timedEvents;
  std::vector<int> timedClass;
  bool curved = false;             // some block curved
  bool facePoint = false;          // some block with per-point face metrics: face geometry per face point
  unsigned waitLimit = 0;          // sdg_set_wait_check: mbarrier wait rounds of the tensor stage kernels
  unsigned txExtra = 0;            // sdg_set_wait_check: bytes declared beyond the tile copies
  bool useGraph = true;            // sdg_step replays a captured CUDA graph of one step
  cudaGraphExec_t graphExec = nullptr;
  double graphDt = 0.0;
  double* pointsOut = nullptr;     // sdg_step_state_point: mapped host buffer the last stage of tensor blocks fills
  double* graphOut = nullptr;      // pointsOut the captured graph was made with
  int64_t graphKernels = 0;
  int64_t elements = 0, dof = 0;
  struct AdjointState* adj = nullptr;  // tangent-linear / adjoint buffers, created on first use
  bool adjointTrajectoryStore = false; // sdg_set_adjoint_trajectory_store: keep every stage input when HBM has room
  uint64_t stateVersion = 0;          // bumped by every call that changes the state or the physics
  std::string err;
};

namespace sdg {
// Launch records of one step (all stages, then the relative-error reduction when `relerr`).
void emitStep(sdg_handle* h, double dt, bool relerr, std::vector<Rec>& out);
// One-instance execution of records on `stream` (kernel timing and launch counting of the handle).
void runRecs(sdg_handle* h, const std::vector<Rec>& recs, cudaStream_t stream);
// Stage kernel record of block B with the handle's buffers (the caller fills the stage fields).
Rec stageRec(sdg_handle* h, DevBlock& B);
Rec gradRec(sdg_handle* h, DevBlock& B, int which);
// Tile shapes.
void setStageTile(DevBlock& B, int slot, int epb, int threads);  // slot: stageV index
void setGradTile(DevBlock& B, int epb, int threads);
void dropGraph(sdg_handle* h);
void traceAll(sdg_handle* h, int which);
void checkStatus(sdg_handle* h);
// Error text returned by sdg_last_error(NULL) (failures before a handle exists).
void setCreateError(const std::string& message);
// Right point of each left point of a triangular interior face per rotation, [3][nfq].
std::vector<int> triangleFacePermutation(int type, int p);
// Face-point record of operation `op` (FaceOp) over the handle's interior or boundary faces.
Rec faceRec(sdg_handle* h, int op);
// SSP-RK coefficients (c0 on the step's base state, c1 on the stage input, c2 on dt R) per scheme and stage.
extern const double kRk[3][3][3];
// Point layout [point][v] <-> state layout of device buffers (tensor: transpose; dense: projection).
void pointsToStateBuffer(sdg_handle* h, const double* pts, double* st);
void stateToPointsBuffer(sdg_handle* h, const double* st, double* pts);
void cotangentPointsToState(sdg_handle* h, const double* pts, double* st);
void cotangentStateToPoints(sdg_handle* h, const double* st, double* pts);
// Tangent-linear / adjoint resources of a handle (sdg_adjoint.cu), released with the handle.
void destroyAdjoint(sdg_handle* h);
// The gradient pass and viscous-layout buffers run for Navier-Stokes and for artificial viscosity.
inline bool viscousPath(const sdg_handle* h) { return h->ns || h->av; }
// Input state of a step's last gradient pass (the last stage's input): the stage buffer for two- and
// three-stage schemes; forward Euler updates in place and keeps none.
inline const double* stepGradientInput(const sdg_handle* h) {
  return h->cfg.time_integration >= 1 ? h->state[1] : nullptr;
}
// The stage-kernel slot of a handle (DevBlock::stageV).
inline int stageSlot(const sdg_handle* h) { return h->av ? 2 : (h->ns ? 1 : 0); }
// Artificial viscosity (sdg_av.cu): inner radius of an element, the block tables, the per-step records.
double innerRadiusOf(int type, const double* nodes, const int32_t* vertices);
void buildAvTables(DevBlock& B);
void emitArtificialViscosity(sdg_handle* h, int seq, std::vector<Rec>& out);
}  // namespace sdg
