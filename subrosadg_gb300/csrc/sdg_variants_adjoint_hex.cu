// Tangent-linear and adjoint element (tile) kernels of hexahedra that are not parallelepipeds (trilinear or
// curved: the metric per node, face metrics per face point), P1..P5: a translation unit of their own so that it
// compiles in parallel with the other kernel families.
#include "sdg_kernels_adjoint.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int N, bool VISC>
void hexOf(AdjointTileKernels& k, bool br2, bool gen) {
  using A = AdjShape<3, N>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpStageKernel<3, N, VISC, false>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpVolumeKernel<3, N, VISC, true, false>)
                    : reinterpret_cast<const void*>(&vjpVolumeKernel<3, N, VISC, false, false>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpTraceKernel<3, N>);
  if constexpr (VISC)
    k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpGradientBilinearKernel<3, N, true>)
                        : reinterpret_cast<const void*>(&vjpGradientBilinearKernel<3, N, false>);
  k.epb = A::EPB; k.threads = A::THREADS; k.jvpSmem = A::JVP_SMEM;
  k.volSmem = A::VOL_SMEM; k.gradSmem = A::GRAD_SMEM; k.traceSmem = A::TRACE_SMEM;
}
template <int N>
void hexOf(AdjointTileKernels& k, bool visc, bool br2, bool gen) {
  if (visc) hexOf<N, true>(k, br2, gen); else hexOf<N, false>(k, false, gen);
}
}  // namespace

void adjointHexNonAffineKernels(int n, bool visc, bool br2, bool gen, AdjointTileKernels& k) {
  switch (n) {
    case 2: hexOf<2>(k, visc, br2, gen); break;
    case 3: hexOf<3>(k, visc, br2, gen); break;
    case 4: hexOf<4>(k, visc, br2, gen); break;
    case 5: hexOf<5>(k, visc, br2, gen); break;
    case 6: hexOf<6>(k, visc, br2, gen); break;
    default: break;
  }
}

}  // namespace sdg
