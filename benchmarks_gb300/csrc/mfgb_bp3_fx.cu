// The FP64-accurate BP3 operator and Gauss p+1 Laplacian with offset
// double-float accumulation (mfgb_bp3fx.cuh; launcher in
// mfgb_bp3fx_launch.cuh), and the CEED BK1 / BK3 E-vector kernels on the same
// arithmetic (mfgb_bk1fx.cuh, mfgb_bk3fx.cuh).
#include <algorithm>
#include <cmath>

#include "mfgb_bk1fx.cuh"
#include "mfgb_bk3fx.cuh"
#include "mfgb_bp3fx_launch.cuh"
#include "mfgb_internal.h"

namespace mfgb {
namespace {

template <int NM, int NQ>
cudaError_t bk1fx_launch(int64_t nelmt, const double *in, const double *JxW, double *out,
                         const double *hB, cudaStream_t s) {
  constexpr int E = Bp3FxElems<NQ>::value, MB = Bp3FxMinBlocks<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  BasisQFX<NM, NQ> b;
  fill_basis(hB, nullptr, b);
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk1fx_kernel<NM, NQ, E, MB>, threads, 0));
  const int64_t batches = (nelmt + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * num_sms()));
  bk1fx_kernel<NM, NQ, E, MB><<<grid, threads, 0, s>>>(nelmt, in, JxW, out, b);
  return cudaGetLastError();
}

template <int NM, int NQ>
cudaError_t bk3fx_launch(int64_t nelmt, const double *G, const double *in, double *out,
                         const double *hB, const double *hDG, cudaStream_t s) {
  constexpr int E = Bp3FxElems<NQ>::value, MB = Bp3FxMinBlocks<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  constexpr size_t smem = TmaLayoutQ<NM, NQ, E, ArithF64, 4>::total;
  BasisQFX<NM, NQ> b;
  fill_basis(hB, hDG, b);
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk3fx_tma_kernel<NM, NQ, E, MB>, threads, smem));
  const int64_t batches = (nelmt + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * num_sms()));
  bk3fx_tma_kernel<NM, NQ, E, MB><<<grid, threads, smem, s>>>(nelmt, G, in, out, b,
                                                               device_error_flag());
  return cudaGetLastError();
}

}  // namespace

cudaError_t bk3_fx(int degree, int64_t nelmt, const double *G, const double *in, double *out,
                   const double *hB, const double *hDG, cudaStream_t s) {
  if (nelmt <= 0) return cudaSuccess;
  if (reinterpret_cast<uintptr_t>(G) & 15u) return cudaErrorInvalidValue;  // bulk copies
  switch (degree) {
#define MFGB_BK3FX(P) \
  case P: return bk3fx_launch<P + 1, P + 2>(nelmt, G, in, out, hB, hDG, s);
    MFGB_BK3FX(1) MFGB_BK3FX(2) MFGB_BK3FX(3) MFGB_BK3FX(4) MFGB_BK3FX(5) MFGB_BK3FX(6)
    MFGB_BK3FX(7) MFGB_BK3FX(8)
#undef MFGB_BK3FX
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t bk1_fx(int degree, int64_t nelmt, const double *in, const double *JxW, double *out,
                   const double *hB, cudaStream_t s) {
  if (nelmt <= 0) return cudaSuccess;
  switch (degree) {
#define MFGB_BK1FX(P) \
  case P: return bk1fx_launch<P + 1, P + 2>(nelmt, in, JxW, out, hB, s);
    MFGB_BK1FX(1) MFGB_BK1FX(2) MFGB_BK1FX(3) MFGB_BK1FX(4) MFGB_BK1FX(5) MFGB_BK1FX(6)
    MFGB_BK1FX(7) MFGB_BK1FX(8)
#undef MFGB_BK1FX
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t bp3_fx(int degree, int nq, int64_t n_cells, const uint32_t *map, const float2 *Gfx,
                   const int *gexp, const double *src, double *dst, const double *hB,
                   const double *hDG, cudaStream_t s, const int *done, const float2 *jxw) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || (reinterpret_cast<uintptr_t>(Gfx) & 15u)) return cudaErrorInvalidValue;
  // bulk copies of the dof-map tiles need a 16-byte aligned map
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  const int extra = nq - degree - 1;  // 1: BP3 (q = p + 2), 0: Gauss p + 1
  if (extra != 0 && extra != 1) return cudaErrorInvalidValue;
  if (jxw != nullptr)  // the Helmholtz form (Gauss p + 1 with the mass term)
    return extra == 0 ? helmholtz_fx(degree, n_cells, map, Gfx, gexp, jxw, src, dst, hB, hDG, s, done)
                      : cudaErrorInvalidValue;
  switch (degree * 2 + extra) {
#define MFGB_BP3FX(P, X)                                                                         \
  case 2 * P + X:                                                                                \
    return mt ? bp3fx_launch<P + 1, P + 1 + X, true>(n_cells, map, Gfx, gexp, src, dst, hB, hDG, s, \
                                                     done, nullptr)                               \
              : bp3fx_launch<P + 1, P + 1 + X, false>(n_cells, map, Gfx, gexp, src, dst, hB, hDG,  \
                                                      s, done, nullptr);
    MFGB_BP3FX(1, 1) MFGB_BP3FX(2, 1) MFGB_BP3FX(3, 1) MFGB_BP3FX(4, 1) MFGB_BP3FX(5, 1)
    MFGB_BP3FX(6, 1) MFGB_BP3FX(7, 1) MFGB_BP3FX(8, 1)
    MFGB_BP3FX(1, 0) MFGB_BP3FX(2, 0) MFGB_BP3FX(3, 0) MFGB_BP3FX(4, 0) MFGB_BP3FX(5, 0)
    MFGB_BP3FX(6, 0) MFGB_BP3FX(7, 0) MFGB_BP3FX(8, 0)
#undef MFGB_BP3FX
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb
