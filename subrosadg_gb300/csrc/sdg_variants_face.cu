// Face-point kernels (Riemann fluxes, boundary fluxes, Navier-Stokes trace exchange, viscous and
// artificial viscous face fluxes) and the relative-error reduction: the one translation unit that
// instantiates them.
#include "sdg_kernels_ns.cuh"
#include "sdg_variants.hpp"

namespace sdg {

__device__ __forceinline__ void relerrReduceBlock(const RelArgs& a, int v) {
  __shared__ double sh[256];
  double acc = 0.0;
  for (int r = 0; r < a.nranges; ++r)
    for (int64_t i = threadIdx.x; i < a.count[r]; i += blockDim.x) acc += a.part[(a.offset[r] + i) * a.nv + v];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.out[v] = sh[0] * a.inv_elements;
}

__global__ void __launch_bounds__(256) relerrReduceKernel(RelArgs a) { relerrReduceBlock(a, blockIdx.x); }

// Batched: blockIdx.y = instance, blockIdx.x = variable.
__global__ void __launch_bounds__(256) relerrReduceBatchKernel(const RelArgs* __restrict__ args) {
  const RelArgs a = args[blockIdx.y];
  if (int(blockIdx.x) < a.nv) relerrReduceBlock(a, blockIdx.x);
}

namespace {
template <int OP, int DIM, int FLUX>
KernelVariant faceOf() {
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&facePointKernel<OP, DIM, FLUX>);
  v.batch = reinterpret_cast<const void*>(&facePointBatchKernel<OP, DIM, FLUX>);
  v.threads = kFaceThreads; v.epb = 1;
  return v;
}
template <int OP, int DIM>
KernelVariant faceFluxOf(int flux) {
  switch (flux) {
    case 0: return faceOf<OP, DIM, 0>();
    case 1: return faceOf<OP, DIM, 1>();
    case 2: return faceOf<OP, DIM, 2>();
    case 3: return faceOf<OP, DIM, 3>();
    case 4: return faceOf<OP, DIM, 4>();
    default: return KernelVariant();
  }
}
template <int DIM>
KernelVariant faceDimOf(int op, int flux) {
  switch (op) {
    case kOpFace: return faceFluxOf<kOpFace, DIM>(flux);
    case kOpFaceBoundary: return faceOf<kOpFaceBoundary, DIM, 0>();
    case kOpExchange: return faceOf<kOpExchange, DIM, 0>();
    case kOpExchangeBoundary: return faceOf<kOpExchangeBoundary, DIM, 0>();
    case kOpFaceNS: return faceFluxOf<kOpFaceNS, DIM>(flux);
    case kOpFaceNSBoundary: return faceOf<kOpFaceNSBoundary, DIM, 0>();
    case kOpFaceAV: return faceFluxOf<kOpFaceAV, DIM>(flux);
    case kOpFaceAVBoundary: return faceOf<kOpFaceAVBoundary, DIM, 0>();
    default: return KernelVariant();
  }
}
}  // namespace

KernelVariant facePointVariant(int op, int dim, int flux) {
  if (dim == 1) return faceDimOf<1>(op, flux);
  if (dim == 2) return faceDimOf<2>(op, flux);
  if (dim == 3) return faceDimOf<3>(op, flux);
  return KernelVariant();
}

KernelVariant relerrVariant() {
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&relerrReduceKernel);
  v.batch = reinterpret_cast<const void*>(&relerrReduceBatchKernel);
  v.threads = 256; v.epb = 1;
  return v;
}

}  // namespace sdg
