// Instantiations of the BK6 (3-component vector Laplacian) kernels.
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"
namespace mfgb {
cudaError_t bk6_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                    const double *src, double *dst, const double *D, cudaStream_t s) {
  return bk6_dispatch<ArithF64>(N, n_cells, map, G, src, dst, D, s);
}
cudaError_t bk6_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const double *src,
                   double *dst, const double *D, cudaStream_t s) {
  return bk6_dispatch<ArithDF>(N, n_cells, map, G, src, dst, D, s);
}
}  // namespace mfgb

namespace {
__global__ void copy_constrained_vec_kernel(int64_t nc, const int64_t *__restrict__ c, int ncomp,
                                            const double *__restrict__ src, double *__restrict__ dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nc * ncomp;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t d = c[t / ncomp] * ncomp + t % ncomp;
    dst[d] = src[d];
  }
}
}  // namespace

using namespace mfgb;

// BK6/BP6 vector Laplacian: ncomp = 3 interleaved FP64 components per DoF
extern "C" mfgb_status mfgb_vmult_vector(const mfgb_operator *cop, double *d_dst,
                                         const double *d_src, int ncomp, int arith, void *stream) {
  if (!cop || ncomp != 3 || (cop->n_dofs > 0 && (!d_dst || !d_src)) || d_dst == d_src ||
      cop->quadrature != 0) {
    set_error("mfgb_vmult_vector: invalid argument (3 components, GLL operator, distinct vectors)");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb_operator *op = const_cast<mfgb_operator *>(cop);
  cudaStream_t s = (cudaStream_t)stream;
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(d_dst, 0, sizeof(double) * 3 * op->n_dofs, s), "dst = 0")))
    return st;
  cudaError_t e;
  if (arith == MFGB_ARITH_FP64) {
    e = bk6_f64(op->n, op->n_cells, op->d_map, op->d_G, d_src, d_dst, op->D, s);
  } else if (arith == MFGB_ARITH_FP64_DF && (op->d_Gfx || op->d_G)) {
    // offset double-float, every component scaled per cell: any input range
    if ((st = ensure_fx(op))) return st;
    e = bk6_fx(op->n, op->n_cells, op->d_map, op->d_Gfx, op->d_Gexp, d_src, d_dst, op->D, s);
  } else if (arith == MFGB_ARITH_FP64_DF) {
    if ((st = ensure_df(op)) || (st = range_check_async(op, 3 * op->n_dofs, d_src, s))) return st;
    e = bk6_df(op->n, op->n_cells, op->d_map, op->d_Gdf, d_src, d_dst, op->D, s);
  } else {
    set_error("mfgb_vmult_vector: unknown arith");
    return MFGB_ERR_INVALID_ARG;
  }
  if ((st = cuda_status(e, "bk6 kernel"))) return st;
  if (op->n_constrained)
    copy_constrained_vec_kernel<<<152 * 8, 256, 0, s>>>(op->n_constrained, op->d_constrained, 3,
                                                        d_src, d_dst);
  return cuda_status(cudaGetLastError(), "bk6 constrained rows");
}
