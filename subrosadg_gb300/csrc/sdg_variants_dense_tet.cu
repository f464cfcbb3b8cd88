// Dense (modal) stage and gradient kernels of tetrahedra, P1..P5: a translation unit of their own so that it
// compiles in parallel with the 2D dense blocks' kernels.
#include "sdg_kernels_dense.cuh"
#include "sdg_kernels_ns.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int NB, int NQ, int NFQ, int NF, int VISC>
KernelVariant stageOf() {
  using S = DenseShape<NB, NQ, NFQ, NF, 3>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&denseStageKernel<NB, NQ, NFQ, NF, true, VISC, 3>);
  v.batch = reinterpret_cast<const void*>(&denseStageBatchKernel<NB, NQ, NFQ, NF, true, VISC, 3>);
  v.nb = NB; v.epb = S::EPB; v.threads = S::THREADS; v.nodeThreads = false;
  v.perElem = size_t(S::PER_ELEM) * 8; v.fixed = S::tables(true) * 8 + 16; v.perWarp = 8 * S::NV;
  return v;
}
template <int NB, int NQ, int NFQ, int NF>
KernelVariant gradOf() {
  using G = DenseGradShape<NB, NQ, NFQ, NF, true, 3>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&denseGradientKernel<NB, NQ, NFQ, NF, true, 3>);
  v.batch = reinterpret_cast<const void*>(&denseGradientBatchKernel<NB, NQ, NFQ, NF, true, 3>);
  v.nb = NB; v.epb = G::EPB; v.threads = G::THREADS; v.nodeThreads = false;
  v.perElem = size_t(G::PER_ELEM) * 8; v.fixed = G::TABLES * 8 + 16; v.perWarp = 0;
  return v;
}
}  // namespace

KernelVariant tetStageVariant(int p, bool affine, int visc) {
#define SDG_DT(T, P, NB, NQ, NFQ, NF)                                                   \
  if (p == P && affine)                                                                 \
    return visc == 2 ? stageOf<NB, NQ, NFQ, NF, 2>()                                    \
                     : visc ? stageOf<NB, NQ, NFQ, NF, 1>() : stageOf<NB, NQ, NFQ, NF, 0>();
  SDG_TET_CASES(SDG_DT)
#undef SDG_DT
  return KernelVariant();
}

KernelVariant tetGradVariant(int p, bool affine) {
#define SDG_DGT(T, P, NB, NQ, NFQ, NF) \
  if (p == P && affine) return gradOf<NB, NQ, NFQ, NF>();
  SDG_TET_CASES(SDG_DGT)
#undef SDG_DGT
  return KernelVariant();
}

}  // namespace sdg
