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

namespace {
template <int DIM>
void boundaryOf(bool visc, AdjointKernels& k) {
  if (!visc) {
    k.jvpBoundary = reinterpret_cast<const void*>(&jvpBoundaryKernel<DIM>);
    k.vjpBoundary = reinterpret_cast<const void*>(&vjpBoundaryKernel<DIM>);
  } else {
    k.jvpBoundary = reinterpret_cast<const void*>(&jvpBoundaryNSKernel<DIM>);
    k.vjpBoundary = reinterpret_cast<const void*>(&vjpBoundaryNSKernel<DIM>);
    k.jvpExchangeBoundary = reinterpret_cast<const void*>(&jvpExchangeBoundaryKernel<DIM>);
    k.vjpExchangeBoundary = reinterpret_cast<const void*>(&vjpExchangeBoundaryKernel<DIM>);
  }
}
template <int DIM>
void dimOf(int flux, bool visc, bool gen, AdjointKernels& k) {
  if (visc) fluxOf<DIM, true>(flux, k, gen); else fluxOf<DIM, false>(flux, k, gen);
  boundaryOf<DIM>(visc, k);
}
}  // namespace

void adjointFaceKernels(int dim, int flux, bool visc, bool gen, AdjointKernels& k) {
  if (dim == 1) dimOf<1>(flux, visc, gen, k);
  else if (dim == 2) dimOf<2>(flux, visc, gen, k);
  else if (dim == 3) dimOf<3>(flux, visc, gen, k);
}

}  // namespace sdg
