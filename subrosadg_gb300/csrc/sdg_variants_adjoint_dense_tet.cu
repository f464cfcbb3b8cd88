// Tangent-linear and adjoint element kernels of tetrahedra (P1..P3): a translation unit of their own so that it
// compiles in parallel with the 2D dense blocks' derivative kernels.
#include "sdg_kernels_adjoint_dense.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
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
}  // namespace

void adjointTetKernels(int p, bool affine, bool gen, bool visc, bool br2, AdjointTileKernels& k) {
#define SDG_ADT(T, P, NB, NQ, NFQ, NF)                     \
  if (p == P && affine) {                                  \
    if (visc) tetOf<NB, NQ, NFQ, NF, true>(k, gen, br2);   \
    else tetOf<NB, NQ, NFQ, NF, false>(k, gen, false);     \
    return;                                                \
  }
  SDG_TET_ADJOINT_CASES(SDG_ADT)
#undef SDG_ADT
}

}  // namespace sdg
