// Tensor-block (lines, quadrangles P>=2, hexahedra) stage and gradient kernels: the one translation unit that
// instantiates them, and their registry entries.
#include "sdg_kernels_ns.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int DIM, int N, bool AFF, int VISC>
KernelVariant stageOf() {
  using S = TensorShape<DIM, N>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&tensorStageKernel<DIM, N, AFF, VISC>);
  v.batch = reinterpret_cast<const void*>(&tensorStageBatchKernel<DIM, N, AFF, VISC>);
  v.nb = S::NB; v.epb = S::EPB; v.threads = S::THREADS; v.nodeThreads = true;
  v.perElem = S::SMEM_PER_ELEM; v.fixed = sizeof(TensorTables) + 16; v.perWarp = 8 * S::NV;
  return v;
}
template <int DIM, int N, bool AFF, bool BR2>
KernelVariant gradOf() {
  using G = GradShape<DIM, N, AFF, BR2>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&tensorGradientKernel<DIM, N, AFF, BR2>);
  v.batch = reinterpret_cast<const void*>(&tensorGradientBatchKernel<DIM, N, AFF, BR2>);
  v.nb = G::NB; v.epb = G::EPB; v.threads = G::THREADS; v.nodeThreads = true;
  v.perElem = size_t(G::PER_ELEM) * 8; v.fixed = sizeof(TensorTables) + 16; v.perWarp = 0;
  return v;
}
}  // namespace

#define SDG_TENSOR_ORDERS(X) \
  X(1, 2) X(1, 3) X(1, 4) X(1, 5) X(1, 6) X(2, 3) X(2, 4) X(2, 5) X(2, 6) X(3, 2) X(3, 3) X(3, 4) X(3, 5) X(3, 6)

KernelVariant tensorStageVariant(int dim, int n, bool affine, int visc) {
#define SDG_TS(D, NN)                                                                                        \
  if (dim == D && n == NN) {                                                                                 \
    if (affine) return visc == 2 ? stageOf<D, NN, true, 2>() : visc ? stageOf<D, NN, true, 1>() : stageOf<D, NN, true, 0>(); \
    if constexpr (D == 2)                                                                                    \
      return visc == 2 ? stageOf<D, NN, false, 2>() : visc ? stageOf<D, NN, false, 1>() : stageOf<D, NN, false, 0>(); \
    if constexpr (D == 3) return hexNonAffineStageVariant(NN, visc);                                         \
    return KernelVariant();                                                                                  \
  }
  SDG_TENSOR_ORDERS(SDG_TS)
#undef SDG_TS
  return KernelVariant();
}

KernelVariant tensorGradVariant(int dim, int n, bool affine, bool br2) {
#define SDG_TG(D, NN)                                                                         \
  if (dim == D && n == NN) {                                                                  \
    if (affine) return br2 ? gradOf<D, NN, true, true>() : gradOf<D, NN, true, false>();       \
    if constexpr (D == 2) return br2 ? gradOf<D, NN, false, true>() : gradOf<D, NN, false, false>(); \
    if constexpr (D == 3) return hexNonAffineGradVariant(NN, br2);                            \
    return KernelVariant();                                                                   \
  }
  SDG_TENSOR_ORDERS(SDG_TG)
#undef SDG_TG
  return KernelVariant();
}

}  // namespace sdg
