// Dense (modal) stage and gradient kernels of 2D blocks (triangles, P1 quadrangles): the translation unit that
// instantiates them, and the registry entries of every dense block (tetrahedra: sdg_variants_dense_tet.cu).
#include "sdg_kernels_dense.cuh"
#include "sdg_kernels_ns.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int NB, int NQ, int NFQ, int NF, bool AFF, int VISC, int DIM = 2>
KernelVariant stageOf() {
  using S = DenseShape<NB, NQ, NFQ, NF, DIM>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&denseStageKernel<NB, NQ, NFQ, NF, AFF, VISC, DIM>);
  v.batch = reinterpret_cast<const void*>(&denseStageBatchKernel<NB, NQ, NFQ, NF, AFF, VISC, DIM>);
  v.nb = NB; v.epb = S::EPB; v.threads = S::THREADS; v.nodeThreads = false;
  v.perElem = size_t(S::PER_ELEM) * 8; v.fixed = S::tables(AFF) * 8 + 16; v.perWarp = 8 * S::NV;
  return v;
}
template <int NB, int NQ, int NFQ, int NF, bool AFF, int DIM = 2>
KernelVariant gradOf() {
  using G = DenseGradShape<NB, NQ, NFQ, NF, AFF, DIM>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&denseGradientKernel<NB, NQ, NFQ, NF, AFF, DIM>);
  v.batch = reinterpret_cast<const void*>(&denseGradientBatchKernel<NB, NQ, NFQ, NF, AFF, DIM>);
  v.nb = NB; v.epb = G::EPB; v.threads = G::THREADS; v.nodeThreads = false;
  v.perElem = size_t(G::PER_ELEM) * 8; v.fixed = G::TABLES * 8 + 16; v.perWarp = 0;
  return v;
}
}  // namespace

KernelVariant denseStageVariant(int type, int p, bool affine, int visc) {
#define SDG_DS(T, P, NB, NQ, NFQ, NF, AFF)                                                                  \
  if (type == T && p == P && affine == AFF)                                                                 \
    return visc == 2 ? stageOf<NB, NQ, NFQ, NF, AFF, 2>()                                                   \
                     : visc ? stageOf<NB, NQ, NFQ, NF, AFF, 1>() : stageOf<NB, NQ, NFQ, NF, AFF, 0>();
  SDG_DENSE_CASES(SDG_DS)
#undef SDG_DS
  if (type == SDG_ELEMENT_TETRAHEDRON) return tetStageVariant(p, affine, visc);
  return KernelVariant();
}

KernelVariant denseGradVariant(int type, int p, bool affine) {
#define SDG_DG(T, P, NB, NQ, NFQ, NF, AFF) \
  if (type == T && p == P && affine == AFF) return gradOf<NB, NQ, NFQ, NF, AFF>();
  SDG_DENSE_CASES(SDG_DG)
#undef SDG_DG
  if (type == SDG_ELEMENT_TETRAHEDRON) return tetGradVariant(p, affine);
  return KernelVariant();
}

}  // namespace sdg
