// Tangent-linear and adjoint element kernels of 2D dense blocks (triangles -- straight or curved --, first-order
// quadrangles -- affine or bilinear --: the Euler and Navier-Stokes (BR1, BR2) equations): the translation unit
// that instantiates them (tetrahedra: sdg_variants_adjoint_dense_tet.cu).
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
  if (type == SDG_ELEMENT_TETRAHEDRON) adjointTetKernels(p, affine, gen, visc, br2, k);
}

}  // namespace sdg
