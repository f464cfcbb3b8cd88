// Kernel variant registry of the GB300 DG path (host side).
//
// Every (element kind, dimension or type, order, affine, viscous) combination is one template
// instantiation of a tile kernel; every (face operation, dimension, flux) one of a face-point kernel.
// Each kernel family is instantiated in exactly one translation unit (sdg_variants_*.cu), which hands
// out the kernel entry points as plain pointers for cudaLaunchKernel, with the shared-memory shape the
// host needs to size a launch for any elements-per-CTA value.  One-instance launches, CUDA-graph
// capture, the batched persistent launches and the autotuner all go through these pointers.
#pragma once
#include <cstddef>
#include <cstdint>

namespace sdg {

struct KernelVariant {
  const void* single = nullptr;   // one CTA per tile / per chunk of points
  const void* batch = nullptr;    // persistent kernel over a work list of (argument set, tile) items
  int nb = 0;                     // nodes (tensor) or basis functions (dense) per element
  int epb = 1;                    // default elements per CTA
  int threads = 256;              // default threads per CTA
  bool nodeThreads = false;       // threads follow epb: one per node, rounded up to whole warps
  size_t perElem = 0, fixed = 0, perWarp = 0;  // dynamic shared memory = epb*perElem + fixed + perWarp*warps
  size_t smem(int e, int t) const { return size_t(e) * perElem + fixed + perWarp * size_t((t + 31) / 32); }
  int threadsFor(int e) const { return nodeThreads ? ((e * nb + 31) / 32) * 32 : threads; }
  bool valid() const { return single != nullptr; }
};

// Tile kernels (elements of one block per CTA).  Unsupported combinations return an invalid variant.
KernelVariant tensorStageVariant(int dim, int n, bool affine, int visc);  // visc: 0 Euler, 1 NS, 2 AV
KernelVariant tensorGradVariant(int dim, int n, bool affine, bool br2);
// Hexahedra that are not parallelepipeds (sdg_variants_tensor_hex.cu), reached through the two above.
KernelVariant hexNonAffineStageVariant(int n, int visc);
KernelVariant hexNonAffineGradVariant(int n, bool br2);
KernelVariant denseStageVariant(int type, int p, bool affine, int visc);
KernelVariant denseGradVariant(int type, int p, bool affine);
// Tetrahedra (sdg_variants_dense_tet.cu), reached through the two above.
KernelVariant tetStageVariant(int p, bool affine, int visc);
KernelVariant tetGradVariant(int p, bool affine);
// Face-point kernels (FaceOp op, flux only for the Riemann operations) and the relative-error reduction.
KernelVariant facePointVariant(int op, int dim, int flux);
KernelVariant relerrVariant();

// Tangent-linear and adjoint face kernels (sdg_kernels_adjoint.cuh), shared by every element block.
struct AdjointKernels {
  const void* jvpFace = nullptr;      // (AdjArgs, Phys), one thread per face point
  const void* vjpFace = nullptr;      // (AdjArgs, Phys), one thread per face point
  const void* vjpExchange = nullptr;  // (AdjArgs), one thread per face point
  const void* jvpBoundary = nullptr;  // (AdjArgs, Phys), one thread per boundary face point
  const void* vjpBoundary = nullptr;  // (AdjArgs, Phys)
  const void* jvpExchangeBoundary = nullptr;  // (AdjArgs, Phys), Navier-Stokes: the gradient pass's wall states
  const void* vjpExchangeBoundary = nullptr;  // (AdjArgs, Phys)
  bool valid() const { return jvpFace && vjpFace; }
};
// Tangent-linear and adjoint element kernels of one block (tensor: sdg_kernels_adjoint.cuh; dense:
// sdg_kernels_adjoint_dense.cuh), one CTA per tile of epb elements.
struct AdjointTileKernels {
  const void* jvpStage = nullptr;     // (AdjArgs, Phys)
  const void* vjpVolume = nullptr;    // (AdjArgs, Phys)
  const void* vjpGradient = nullptr;  // (AdjArgs), Navier-Stokes
  const void* vjpTrace = nullptr;     // (AdjArgs)
  int epb = 0, threads = 0;
  size_t jvpSmem = 0, volSmem = 0, gradSmem = 0, traceSmem = 0;  // dynamic shared memory of each kernel
  bool valid() const { return jvpStage && vjpVolume && vjpTrace; }
};
// Face kernels depend on (dim, flux, viscous); tensor tile kernels on (dim, nodes per direction, viscous, BR2,
// affine: bilinear quadrangles for the Euler equations only); dense tile kernels on (type, order, affine,
// viscous, BR2: Navier-Stokes on affine elements).  gen: the dual-number transposes (incompressible model,
// Boussinesq source) instead of the hand-written ones.  Unsupported combinations leave the kernels null.
void adjointFaceKernels(int dim, int flux, bool visc, bool gen, AdjointKernels& k);
void adjointTileKernels(int dim, int n, bool visc, bool br2, bool gen, bool affine, AdjointTileKernels& k);
void adjointDenseKernels(int type, int p, bool affine, bool gen, bool visc, bool br2, AdjointTileKernels& k);
// Tetrahedra (sdg_variants_adjoint_dense_tet.cu), reached through adjointDenseKernels.
void adjointTetKernels(int p, bool affine, bool gen, bool visc, bool br2, AdjointTileKernels& k);
// Hexahedra that are not parallelepipeds (sdg_variants_adjoint_hex.cu), reached through adjointTileKernels.
void adjointHexNonAffineKernels(int n, bool visc, bool br2, bool gen, AdjointTileKernels& k);

// Largest tile size the kernels are compiled for (their __launch_bounds__).
constexpr int kMaxThreads = 512;

}  // namespace sdg
