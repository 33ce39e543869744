// Instantiations of the BK5 kernels with double-float arithmetic on the FP32 pipes.
// (The kernels' per-CTA energy output, WITH_ENERGY, is not instantiated: no
// caller asks for it; a non-null `partials` is refused.)
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"
namespace mfgb {
cudaError_t bk5_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const double *src,
                   double *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                   const int *done) {
  if (partials) return cudaErrorNotSupported;
  return bk5_dispatch<ArithDF, false, false>(N, n_cells, map, G, src, dst, D, nullptr, grid, s,
                                             done);
}
cudaError_t bk5_df_g64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                       const double *src, double *dst, const double *D, cudaStream_t s,
                       const int *done) {
  if (map == nullptr)
    return bk5_dispatch<ArithDFG64, true, false>(N, n_cells, map, G, src, dst, D, nullptr, nullptr, s);
  return bk5_dispatch<ArithDFG64, false, false>(N, n_cells, map, G, src, dst, D, nullptr, nullptr, s,
                                                done);
}
}  // namespace mfgb
