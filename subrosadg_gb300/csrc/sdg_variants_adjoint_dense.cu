// Tangent-linear and adjoint element kernels of dense blocks (triangles, first-order quadrangles), the Euler
// equations: the one translation unit that instantiates them.
#include "sdg_kernels_adjoint_dense.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int NB, int NQ, int NFQ, int NF, bool AFF>
void denseOf(AdjointTileKernels& k, bool gen) {
  using S = DenseAdjShape<NB, NQ, NFQ, NF>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpDenseStageKernel<NB, NQ, NFQ, NF, AFF>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, AFF, true>)
                    : reinterpret_cast<const void*>(&vjpDenseVolumeKernel<NB, NQ, NFQ, NF, AFF, false>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpDenseTraceKernel<NB, NQ, NFQ, NF>);
  k.epb = S::EPB; k.threads = S::THREADS; k.jvpSmem = S::JVP_SMEM; k.volSmem = S::VJP_SMEM;
  k.traceSmem = S::TRACE_SMEM;
}
}  // namespace

void adjointDenseKernels(int type, int p, bool affine, bool gen, AdjointTileKernels& k) {
#define SDG_AD(T, P, NB, NQ, NFQ, NF, AFF) \
  if (type == T && p == P && affine == AFF) { denseOf<NB, NQ, NFQ, NF, AFF>(k, gen); return; }
  SDG_DENSE_CASES(SDG_AD)
#undef SDG_AD
}

}  // namespace sdg
