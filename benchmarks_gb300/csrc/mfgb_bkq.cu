// mfgb_bkq.cu -- C ABI of the CEED BK1 / BK3 E-vector seams (nq = p + 2).
#include <algorithm>
#include <string>

#include "mfgb_bkq.cuh"
#include "mfgb_dispatch.cuh"
#include "mfgb_internal.h"

namespace mfgb {
namespace {

template <int NM, int NQ, class A, bool LAPLACE>
cudaError_t bkq_launch(int64_t nelmt, const double *basis, const double *dbasis, const double *coef,
                       const double *in, double *out, cudaStream_t s, const uint32_t *map) {
  constexpr int E = BkqElems<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  static int per_sm = -1;
  if (per_sm < 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bkq_kernel<NM, NQ, A, LAPLACE>,
                                                      threads, 0) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t batches = (nelmt + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * sms));
  bkq_kernel<NM, NQ, A, LAPLACE><<<grid, threads, 0, s>>>(nelmt, basis, dbasis, coef, in, out,
                                                           map);
  return cudaGetLastError();
}

template <class A, bool LAPLACE>
cudaError_t bkq_dispatch(int degree, int64_t nelmt, const double *basis, const double *dbasis,
                         const double *coef, const double *in, double *out, cudaStream_t s,
                         const uint32_t *map = nullptr) {
  switch (degree) {
    case 1: return bkq_launch<2, 3, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 2: return bkq_launch<3, 4, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 3: return bkq_launch<4, 5, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 4: return bkq_launch<5, 6, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 5: return bkq_launch<6, 7, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 6: return bkq_launch<7, 8, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 7: return bkq_launch<8, 9, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    case 8: return bkq_launch<9, 10, A, LAPLACE>(nelmt, basis, dbasis, coef, in, out, s, map);
    default: return cudaErrorInvalidValue;
  }
}

mfgb_status bkq_entry(const char *name, bool laplace, int degree, int64_t nelmt,
                      const double *basis, const double *dbasis, const double *coef,
                      const double *in, double *out, int arith, void *stream) {
  if (degree < 1 || degree > 8 || nelmt < 0 || (nelmt > 0 && (!basis || !coef || !in || !out)) ||
      (laplace && nelmt > 0 && !dbasis) ||
      (arith != MFGB_ARITH_FP64 && arith != MFGB_ARITH_FP64_DF && arith != MFGB_ARITH_FP64_TC)) {
    set_error(std::string(name) + ": invalid argument (degree 1..8, arith FP64, FP64_DF or FP64_TC)");
    return MFGB_ERR_INVALID_ARG;
  }
  if (arith == MFGB_ARITH_FP64_TC && (laplace || degree > 6)) {
    set_error(std::string(name) + ": FP64_TC is the BK1 mass operator at degree 1..6");
    return MFGB_ERR_UNSUPPORTED;
  }
  if (nelmt == 0) return MFGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (arith == MFGB_ARITH_FP64_TC)
    return cuda_status(bk1_dmma(degree, nelmt, basis, coef, in, out, s), name);
  if (arith == MFGB_ARITH_FP64_DF &&
      (!laplace || (reinterpret_cast<uintptr_t>(coef) & 15u) == 0)) {
    // offset double-float with per-element scaling: any input range, no check
    // (the BK3 kernel's bulk copies of G need a 16-byte aligned array)
    const int nm = degree + 1, nq = degree + 2;
    double hB[100], hD[100];
    mfgb_status st = cuda_status(cudaMemcpyAsync(hB, basis, sizeof(double) * nq * nm,
                                                 cudaMemcpyDeviceToHost, s),
                                 "basis");
    if (!st && laplace)
      st = cuda_status(cudaMemcpyAsync(hD, dbasis, sizeof(double) * nq * nq,
                                       cudaMemcpyDeviceToHost, s),
                       "derivative");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "basis");
    if (st) return st;
    return cuda_status(laplace ? bk3_fx(degree, nelmt, coef, in, out, hB, hD, s)
                               : bk1_fx(degree, nelmt, in, coef, out, hB, s),
                       name);
  }
  if (arith == MFGB_ARITH_FP64_DF) {
    // the double-float range of the inputs and of the caller's coefficients,
    // reported through the device error word (mfgb_check_device_errors)
    const int nm = degree + 1, nq = degree + 2;
    int *slot = nullptr;
    mfgb_status st = cuda_status(cudaMallocAsync((void **)&slot, sizeof(int), s), "range slot");
    if (!st) st = vec_range_check(slot, nelmt * nm * nm * nm, in, s);
    if (slot) cudaFreeAsync(slot, s);
    if (!st) st = cells_range_check(nelmt, (laplace ? 6 : 1) * nq * nq * nq, coef, s);
    if (st) return st;
  }
  if (arith == MFGB_ARITH_FP64)
    e = laplace ? bkq_dispatch<ArithF64, true>(degree, nelmt, basis, dbasis, coef, in, out, s)
                : bkq_dispatch<ArithF64, false>(degree, nelmt, basis, dbasis, coef, in, out, s);
  else
    e = laplace ? bkq_dispatch<ArithDF, true>(degree, nelmt, basis, dbasis, coef, in, out, s)
                : bkq_dispatch<ArithDF, false>(degree, nelmt, basis, dbasis, coef, in, out, s);
  return cuda_status(e, name);
}

}  // namespace

namespace {

// cells per CTA of the BP3 TMA kernel: about 7 warps of NQ^2-thread cells
template <int NQ> struct Bp3Elems {
  static constexpr int value =
      NQ == 3 ? 24 : NQ == 4 ? 14 : NQ == 5 ? 9 : NQ == 6 ? 6 : NQ == 7 ? 4 : NQ <= 9 ? 2 : 1;
};
// residency: 2 CTAs per SM (128 registers a thread) up to NQ = 6, else 1
template <int NQ> struct Bp3MinBlocks { static constexpr int value = NQ <= 6 ? 2 : 1; };

template <int NM, int NQ, class A>
cudaError_t bp3_tma_launch(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                           const double *src, double *dst, const double *hB, const double *hDG,
                           cudaStream_t s) {
  constexpr int E = Bp3Elems<NQ>::value;
  constexpr int MB = Bp3MinBlocks<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  constexpr size_t smem = TmaLayoutQ<NM, NQ, E, A, 4>::total;
  BasisQ<NM, NQ, A> basis;
  for (int q = 0; q < NQ * NM; ++q) basis.B[q] = BasisValue<A>::from(hB[q]);
  for (int q = 0; q < NQ * NQ; ++q) basis.D[q] = BasisValue<A>::from(hDG[q]);
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bp3_tma_kernel<NM, NQ, E, A, MB>, threads, smem));
  const int64_t batches = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * num_sms()));
  bp3_tma_kernel<NM, NQ, E, A, MB><<<grid, threads, smem, s>>>(n_cells, map, G, src, dst, basis,
                                                                 device_error_flag());
  return cudaGetLastError();
}

template <class A>
cudaError_t bp3_tma_dispatch(int degree, int64_t n_cells, const uint32_t *map,
                             const typename A::GType *G, const double *src, double *dst,
                             const double *hB, const double *hDG, cudaStream_t s) {
  switch (degree) {
#define MFGB_BP3(P) \
  case P: return bp3_tma_launch<P + 1, P + 2, A>(n_cells, map, G, src, dst, hB, hDG, s);
    MFGB_BP3(1) MFGB_BP3(2) MFGB_BP3(3) MFGB_BP3(4) MFGB_BP3(5) MFGB_BP3(6) MFGB_BP3(7) MFGB_BP3(8)
#undef MFGB_BP3
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// BP3 operator apply: dst += A src over n_cells cells (gather / scatter through
// map).  16-byte aligned G and map run the bulk-TMA kernel (G as FP64 or as
// double-float pairs, Gdf); otherwise the line kernel bkq_kernel with FP64 G.
cudaError_t bp3_apply(int degree, int64_t n_cells, const uint32_t *map, const double *d_B,
                      const double *d_DG, const double *h_B, const double *h_DG, const double *G,
                      const float2 *Gdf, const double *src, double *dst, int arith,
                      cudaStream_t s) {
  if (n_cells <= 0) return cudaSuccess;
  const bool f64 = arith == MFGB_ARITH_FP64;
  const uintptr_t g = f64 ? reinterpret_cast<uintptr_t>(G) : reinterpret_cast<uintptr_t>(Gdf);
  if (g != 0 && ((g | reinterpret_cast<uintptr_t>(map)) & 15u) == 0)
    return f64 ? bp3_tma_dispatch<ArithF64>(degree, n_cells, map, G, src, dst, h_B, h_DG, s)
               : bp3_tma_dispatch<ArithDF>(degree, n_cells, map, Gdf, src, dst, h_B, h_DG, s);
  return f64 ? bkq_dispatch<ArithF64, true>(degree, n_cells, d_B, d_DG, G, src, dst, s, map)
             : bkq_dispatch<ArithDF, true>(degree, n_cells, d_B, d_DG, G, src, dst, s, map);
}

}  // namespace mfgb

using namespace mfgb;

extern "C" {

mfgb_status mfgb_bk1_evector(int degree, int64_t nelmt, const double *d_basis, const double *d_JxW,
                             const double *d_in, double *d_out, int arith, void *stream) {
  return bkq_entry("mfgb_bk1_evector", false, degree, nelmt, d_basis, nullptr, d_JxW, d_in, d_out,
                   arith, stream);
}

mfgb_status mfgb_bk3_evector(int degree, int64_t nelmt, const double *d_basis,
                             const double *d_dbasis, const double *d_G, const double *d_in,
                             double *d_out, int arith, void *stream) {
  return bkq_entry("mfgb_bk3_evector", true, degree, nelmt, d_basis, d_dbasis, d_G, d_in, d_out,
                   arith, stream);
}

}  // extern "C"
