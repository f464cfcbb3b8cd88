// Tensor-block stage and gradient kernels of hexahedra that are not parallelepipeds (trilinear or curved:
// the metric |J| dxi/dx and 1/|J| per node, face metrics per face point), P1..P5.  A translation unit of
// their own so that it compiles in parallel with the other kernel families.
#include "sdg_kernels_ns.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int N, int VISC>
KernelVariant stageOf() {
  using S = TensorShape<3, N>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&tensorStageKernel<3, N, false, VISC>);
  v.batch = reinterpret_cast<const void*>(&tensorStageBatchKernel<3, N, false, VISC>);
  v.nb = S::NB; v.epb = S::EPB; v.threads = S::THREADS; v.nodeThreads = true;
  v.perElem = S::SMEM_PER_ELEM; v.fixed = sizeof(TensorTables) + 16; v.perWarp = 8 * S::NV;
  return v;
}
template <int N, bool BR2>
KernelVariant gradOf() {
  using G = GradShape<3, N, false, BR2>;
  KernelVariant v;
  v.single = reinterpret_cast<const void*>(&tensorGradientKernel<3, N, false, BR2>);
  v.batch = reinterpret_cast<const void*>(&tensorGradientBatchKernel<3, N, false, BR2>);
  v.nb = G::NB; v.epb = G::EPB; v.threads = G::THREADS; v.nodeThreads = true;
  v.perElem = size_t(G::PER_ELEM) * 8; v.fixed = sizeof(TensorTables) + 16; v.perWarp = 0;
  return v;
}
}  // namespace

#define SDG_HEX_ORDERS(X) X(2) X(3) X(4) X(5) X(6)

KernelVariant hexNonAffineStageVariant(int n, int visc) {
#define SDG_HS(NN) \
  if (n == NN) return visc == 2 ? stageOf<NN, 2>() : visc ? stageOf<NN, 1>() : stageOf<NN, 0>();
  SDG_HEX_ORDERS(SDG_HS)
#undef SDG_HS
  return KernelVariant();
}

KernelVariant hexNonAffineGradVariant(int n, bool br2) {
#define SDG_HG(NN) \
  if (n == NN) return br2 ? gradOf<NN, true>() : gradOf<NN, false>();
  SDG_HEX_ORDERS(SDG_HG)
#undef SDG_HG
  return KernelVariant();
}

}  // namespace sdg
