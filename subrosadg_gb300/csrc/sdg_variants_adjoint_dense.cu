// Tangent-linear and adjoint element kernels of dense blocks (triangles, first-order quadrangles -- affine or
// bilinear --, tetrahedra: the Euler and Navier-Stokes (BR1, BR2) equations): the one
// translation unit that instantiates them.
#include "sdg_kernels_adjoint_dense.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int NB, int NQ, int NFQ, int NF, bool AFF, bool VISC>
void denseOf(AdjointTileKernels& k, bool gen, bool br2) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpDenseStageKernel<NB, NQ, NFQ, NF, AFF, VISC>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, AFF, true, VISC>)
                    : reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, AFF, false, VISC>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpDenseTraceKernel<NB, NQ, NFQ, NF>);
  if constexpr (VISC && AFF) {
    k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpDenseGradientKernel<NB, NQ, NFQ, NF, true>)
                        : reinterpret_cast<const void*>(&vjpDenseGradientKernel<NB, NQ, NFQ, NF, false>);
    k.gradSmem = S::GRAD_SMEM;
  } else if constexpr (VISC) {
    k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpDenseGradientGeneralKernel<NB, NQ, NFQ, NF, true>)
                        : reinterpret_cast<const void*>(&vjpDenseGradientGeneralKernel<NB, NQ, NFQ, NF, false>);
    k.gradSmem = S::GRAD_GENERAL_SMEM;
  }
  k.epb = S::EPB; k.threads = S::THREADS; k.jvpSmem = S::JVP_SMEM; k.volSmem = S::VJP_SMEM;
  k.traceSmem = S::TRACE_SMEM;
}
// Tetrahedra (DIM 3, affine): the Euler and Navier-Stokes (BR1, BR2) equations, compressible and incompressible.
template <int NB, int NQ, int NFQ, int NF, bool VISC>
void tetOf(AdjointTileKernels& k, bool gen, bool br2) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF, 3>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpDenseStageKernel<NB, NQ, NFQ, NF, true, VISC, 3>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, true, true, VISC, 3>)
                    : reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, true, false, VISC, 3>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpDenseTraceKernel<NB, NQ, NFQ, NF, 3>);
  if constexpr (VISC) {
    k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpDenseGradientKernel<NB, NQ, NFQ, NF, true, 3>)
                        : reinterpret_cast<const void*>(&vjpDenseGradientKernel<NB, NQ, NFQ, NF, false, 3>);
    k.gradSmem = S::GRAD_SMEM;
  }
  k.epb = S::EPB; k.threads = S::THREADS; k.jvpSmem = S::JVP_SMEM; k.volSmem = S::VJP_SMEM;
  k.traceSmem = S::TRACE_SMEM;
}
template <int NB, int NQ, int NFQ, int NF, bool AFF>
void denseOf(AdjointTileKernels& k, bool gen, bool visc, bool br2) {
  if (visc) denseOf<NB, NQ, NFQ, NF, AFF, true>(k, gen, br2);
  else denseOf<NB, NQ, NFQ, NF, AFF, false>(k, gen, false);
}
}  // namespace

void adjointDenseKernels(int type, int p, bool affine, bool gen, bool visc, bool br2, AdjointTileKernels& k) {
#define SDG_AD(T, P, NB, NQ, NFQ, NF, AFF) \
  if (type == T && p == P && affine == AFF) { denseOf<NB, NQ, NFQ, NF, AFF>(k, gen, visc, br2); return; }
  SDG_DENSE_ADJOINT_CASES(SDG_AD)
#undef SDG_AD
#define SDG_ADT(T, P, NB, NQ, NFQ, NF) \
  if (type == T && p == P && affine) {                                                   \
    if (visc) tetOf<NB, NQ, NFQ, NF, true>(k, gen, br2);                                 \
    else tetOf<NB, NQ, NFQ, NF, false>(k, gen, false);                                   \
    return;                                                                              \
  }
  SDG_TET_ADJOINT_CASES(SDG_ADT)
#undef SDG_ADT
}

}  // namespace sdg
