// The Helmholtz operator of bp5_kokkos (mass + stiffness at QGauss(p+1);
// reference bp5_kokkos/benchmark.cc:51-251) on the Gauss-point
// offset-accumulation kernel with its mass term (mfgb_bp3fx.cuh, MASS = true):
// the instantiations, in their own translation unit for a parallel build.
#include "mfgb_bp3fx_launch.cuh"
#include "mfgb_internal.h"

namespace mfgb {

cudaError_t helmholtz_fx(int degree, int64_t n_cells, const uint32_t *map, const float2 *Gfx,
                         const int *gexp, const float2 *jxw, const double *src, double *dst,
                         const double *hB, const double *hDG, cudaStream_t s, const int *done) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || jxw == nullptr || (reinterpret_cast<uintptr_t>(Gfx) & 15u))
    return cudaErrorInvalidValue;
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  switch (degree) {
#define MFGB_HFX(P)                                                                             \
  case P:                                                                                       \
    return mt ? bp3fx_launch<P + 1, P + 1, true, true>(n_cells, map, Gfx, gexp, src, dst, hB,   \
                                                       hDG, s, done, jxw)                       \
              : bp3fx_launch<P + 1, P + 1, false, true>(n_cells, map, Gfx, gexp, src, dst, hB,  \
                                                        hDG, s, done, jxw);
    MFGB_HFX(1) MFGB_HFX(2) MFGB_HFX(3) MFGB_HFX(4) MFGB_HFX(5) MFGB_HFX(6) MFGB_HFX(7) MFGB_HFX(8)
#undef MFGB_HFX
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb
