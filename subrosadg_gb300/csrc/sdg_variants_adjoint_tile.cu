// Tangent-linear and adjoint element (tile) kernels of affine tensor blocks (lines, quadrangles, hexahedra): the one translation unit that
// instantiates them.
#include "sdg_kernels_adjoint.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int DIM, int N, bool VISC>
void tileOf(AdjointKernels& k, bool br2, bool gen) {
  using A = AdjShape<DIM, N>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpStageKernel<DIM, N, VISC>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpVolumeKernel<DIM, N, VISC, true>)
                    : reinterpret_cast<const void*>(&vjpVolumeKernel<DIM, N, VISC, false>);
  k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpGradientBR2Kernel<DIM, N>)
                      : reinterpret_cast<const void*>(&vjpGradientKernel<DIM, N>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpTraceKernel<DIM, N>);
  k.epb = A::EPB; k.threads = A::THREADS; k.jvpSmem = A::JVP_SMEM; k.vjpSmem = A::VJP_SMEM;
}
}  // namespace

void adjointTileKernels(int dim, int n, bool visc, bool br2, bool gen, AdjointKernels& k) {
#define SDG_AT(D, NN) \
  if (dim == D && n == NN) { if (visc) tileOf<D, NN, true>(k, br2, gen); else tileOf<D, NN, false>(k, false, gen); return; }
  SDG_AT(1, 2) SDG_AT(1, 3) SDG_AT(1, 4) SDG_AT(1, 5) SDG_AT(1, 6)
  SDG_AT(2, 3) SDG_AT(2, 4) SDG_AT(2, 5) SDG_AT(2, 6) SDG_AT(3, 2) SDG_AT(3, 3) SDG_AT(3, 4) SDG_AT(3, 5) SDG_AT(3, 6)
#undef SDG_AT
}

}  // namespace sdg
