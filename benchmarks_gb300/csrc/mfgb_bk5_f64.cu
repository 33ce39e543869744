// Instantiations of the BK5 kernels with native FP64 arithmetic.
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"
namespace mfgb {
cudaError_t bk5_f64(int N, int64_t n_cells, const uint32_t *map, const double *G, const double *src,
                    double *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                    const int *done) {
  if (partials) return cudaErrorNotSupported;
  if (map == nullptr)
    return bk5_dispatch<ArithF64, true, false>(N, n_cells, map, G, src, dst, D, nullptr, grid, s);
  return bk5_dispatch<ArithF64, false, false>(N, n_cells, map, G, src, dst, D, nullptr, grid, s,
                                              done);
}
}  // namespace mfgb
