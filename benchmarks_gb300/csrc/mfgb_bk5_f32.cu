// Instantiations of the BK5 kernels with FP32 arithmetic and FP32 vectors.
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"
namespace mfgb {
cudaError_t bk5_f32(int N, int64_t n_cells, const uint32_t *map, const float *G, const float *src,
                    float *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                    const int *done) {
  if (partials) return cudaErrorNotSupported;
  return bk5_dispatch<ArithF32, false, false>(N, n_cells, map, G, src, dst, D, nullptr, grid, s,
                                              done);
}
}  // namespace mfgb
