// Instantiations of the Gauss-quadrature (BP5-variant) operator kernels.
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"
namespace mfgb {
cudaError_t bk5g_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                     const double *src, double *dst, const double *DG, const double *B,
                     double *partials, int *grid, cudaStream_t s, const int *done,
                     const double *jxw) {
  if (partials) return cudaErrorNotSupported;
  return bk5g_dispatch<ArithF64, false>(N, n_cells, map, G, src, dst, DG, B, nullptr, grid, s, done,
                                        jxw);
}
cudaError_t bk5g_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G,
                    const double *src, double *dst, const double *DG, const double *B,
                    double *partials, int *grid, cudaStream_t s, const int *done,
                    const float2 *jxw) {
  if (partials) return cudaErrorNotSupported;
  return bk5g_dispatch<ArithDF, false>(N, n_cells, map, G, src, dst, DG, B, nullptr, grid, s, done,
                                       jxw);
}
}  // namespace mfgb
