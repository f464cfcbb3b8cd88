// Tangent-linear and adjoint element (tile) kernels of tensor blocks (lines, quadrangles -- affine or bilinear --,
// hexahedra): the one translation unit that
// instantiates them.
#include "sdg_kernels_adjoint.cuh"
#include "sdg_variants.hpp"

namespace sdg {

namespace {
template <int DIM, int N, bool VISC>
void tileOf(AdjointTileKernels& k, bool br2, bool gen) {
  using A = AdjShape<DIM, N>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpStageKernel<DIM, N, VISC>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpVolumeKernel<DIM, N, VISC, true>)
                    : reinterpret_cast<const void*>(&vjpVolumeKernel<DIM, N, VISC, false>);
  k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpGradientBR2Kernel<DIM, N>)
                      : reinterpret_cast<const void*>(&vjpGradientKernel<DIM, N>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpTraceKernel<DIM, N>);
  k.epb = A::EPB; k.threads = A::THREADS; k.jvpSmem = A::JVP_SMEM;
  k.volSmem = A::VOL_SMEM; k.gradSmem = A::GRAD_SMEM; k.traceSmem = A::TRACE_SMEM;
}
// Bilinear quadrangles (per-node metric): the Euler equations and Navier-Stokes BR1 / BR2.
template <int N, bool VISC>
void bilinearOf(AdjointTileKernels& k, bool br2, bool gen) {
  using A = AdjShape<2, N>;
  k.jvpStage = reinterpret_cast<const void*>(&jvpStageKernel<2, N, VISC, false>);
  k.vjpVolume = gen ? reinterpret_cast<const void*>(&vjpVolumeKernel<2, N, VISC, true, false>)
                    : reinterpret_cast<const void*>(&vjpVolumeKernel<2, N, VISC, false, false>);
  k.vjpTrace = reinterpret_cast<const void*>(&vjpTraceKernel<2, N>);
  if constexpr (VISC)
    k.vjpGradient = br2 ? reinterpret_cast<const void*>(&vjpGradientBilinearKernel<2, N, true>)
                        : reinterpret_cast<const void*>(&vjpGradientBilinearKernel<2, N, false>);
  k.epb = A::EPB; k.threads = A::THREADS; k.jvpSmem = A::JVP_SMEM;
  k.volSmem = A::VOL_SMEM; k.gradSmem = A::GRAD_SMEM; k.traceSmem = A::TRACE_SMEM;
}
template <int N>
void bilinearOf(AdjointTileKernels& k, bool visc, bool br2, bool gen) {
  if (visc) bilinearOf<N, true>(k, br2, gen); else bilinearOf<N, false>(k, false, gen);
}
}  // namespace

void adjointTileKernels(int dim, int n, bool visc, bool br2, bool gen, bool affine, AdjointTileKernels& k) {
  if (!affine) {
    if (dim == 3) { adjointHexNonAffineKernels(n, visc, br2, gen, k); return; }
    if (dim != 2) return;
    switch (n) {
      case 3: bilinearOf<3>(k, visc, br2, gen); break;
      case 4: bilinearOf<4>(k, visc, br2, gen); break;
      case 5: bilinearOf<5>(k, visc, br2, gen); break;
      case 6: bilinearOf<6>(k, visc, br2, gen); break;
      default: break;
    }
    return;
  }
#define SDG_AT(D, NN) \
  if (dim == D && n == NN) { if (visc) tileOf<D, NN, true>(k, br2, gen); else tileOf<D, NN, false>(k, false, gen); return; }
  SDG_AT(1, 2) SDG_AT(1, 3) SDG_AT(1, 4) SDG_AT(1, 5) SDG_AT(1, 6)
  SDG_AT(2, 3) SDG_AT(2, 4) SDG_AT(2, 5) SDG_AT(2, 6) SDG_AT(3, 2) SDG_AT(3, 3) SDG_AT(3, 4) SDG_AT(3, 5) SDG_AT(3, 6)
#undef SDG_AT
}

}  // namespace sdg
