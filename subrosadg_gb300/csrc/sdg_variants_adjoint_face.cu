// Tangent-linear and adjoint face kernels (interior and boundary faces): the one translation unit that instantiates
// them.
#include "sdg_kernels_adjoint.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int DIM, int FLUX, bool VISC>
void faceOf(AdjointKernels& k) {
  k.jvpFace = reinterpret_cast<const void*>(&jvpFaceKernel<DIM, FLUX, VISC>);
  k.vjpFace = reinterpret_cast<const void*>(&vjpFaceKernel<DIM, FLUX, VISC>);
  k.vjpExchange = reinterpret_cast<const void*>(&vjpExchangeKernel<DIM>);
}
template <int DIM, bool VISC>
void fluxOf(int flux, AdjointKernels& k) {
  switch (flux) {
    case 0: faceOf<DIM, 0, VISC>(k); break;
    case 1: faceOf<DIM, 1, VISC>(k); break;
    case 2: faceOf<DIM, 2, VISC>(k); break;
    case 3: faceOf<DIM, 3, VISC>(k); break;
    default: break;
  }
}
}  // namespace

void adjointFaceKernels(int dim, int flux, bool visc, AdjointKernels& k) {
  if (dim == 2) { if (visc) fluxOf<2, true>(flux, k); else fluxOf<2, false>(flux, k); }
  else if (dim == 3) { if (visc) fluxOf<3, true>(flux, k); else fluxOf<3, false>(flux, k); }
  const auto pick = [dim](const void* two, const void* three) { return dim == 2 ? two : three; };
  if (!visc) {
    k.jvpBoundary = pick(reinterpret_cast<const void*>(&jvpBoundaryKernel<2>), reinterpret_cast<const void*>(&jvpBoundaryKernel<3>));
    k.vjpBoundary = pick(reinterpret_cast<const void*>(&vjpBoundaryKernel<2>), reinterpret_cast<const void*>(&vjpBoundaryKernel<3>));
  } else {
    k.jvpBoundary = pick(reinterpret_cast<const void*>(&jvpBoundaryNSKernel<2>), reinterpret_cast<const void*>(&jvpBoundaryNSKernel<3>));
    k.vjpBoundary = pick(reinterpret_cast<const void*>(&vjpBoundaryNSKernel<2>), reinterpret_cast<const void*>(&vjpBoundaryNSKernel<3>));
    k.jvpExchangeBoundary = pick(reinterpret_cast<const void*>(&jvpExchangeBoundaryKernel<2>),
                                 reinterpret_cast<const void*>(&jvpExchangeBoundaryKernel<3>));
    k.vjpExchangeBoundary = pick(reinterpret_cast<const void*>(&vjpExchangeBoundaryKernel<2>),
                                 reinterpret_cast<const void*>(&vjpExchangeBoundaryKernel<3>));
  }
}

}  // namespace sdg
