// Tangent-linear and adjoint face kernels (interior and boundary faces): the one translation unit that instantiates
// them.
#include "sdg_kernels_adjoint.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int DIM, int FLUX, bool VISC>
void faceOf(AdjointKernels& k, bool gen) {
  k.jvpFace = reinterpret_cast<const void*>(&jvpFaceKernel<DIM, FLUX, VISC>);
  k.vjpFace = gen && VISC ? reinterpret_cast<const void*>(&vjpFaceKernel<DIM, FLUX, VISC, VISC>)
                          : reinterpret_cast<const void*>(&vjpFaceKernel<DIM, FLUX, VISC, false>);
  k.vjpExchange = reinterpret_cast<const void*>(&vjpExchangeKernel<DIM>);
}
template <int DIM, bool VISC>
void fluxOf(int flux, AdjointKernels& k, bool gen) {
  switch (flux) {
    case 0: faceOf<DIM, 0, VISC>(k, gen); break;
    case 1: faceOf<DIM, 1, VISC>(k, gen); break;
    case 2: faceOf<DIM, 2, VISC>(k, gen); break;
    case 3: faceOf<DIM, 3, VISC>(k, false); break;   // Roe: compressible only
    case 4: faceOf<DIM, 4, VISC>(k, gen); break;
    default: break;
  }
}
}  // namespace

void adjointFaceKernels(int dim, int flux, bool visc, bool gen, AdjointKernels& k) {
  if (dim == 2) { if (visc) fluxOf<2, true>(flux, k, gen); else fluxOf<2, false>(flux, k, gen); }
  else if (dim == 3) { if (visc) fluxOf<3, true>(flux, k, gen); else fluxOf<3, false>(flux, k, gen); }
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
