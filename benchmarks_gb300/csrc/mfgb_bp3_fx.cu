// The FP64-accurate BP3 operator and Gauss p+1 Laplacian with offset
// double-float accumulation (mfgb_bp3fx.cuh): basis split and bound factors,
// launcher.
#include <algorithm>
#include <cmath>

#include "mfgb_bk1fx.cuh"
#include "mfgb_bk3fx.cuh"
#include "mfgb_bp3fx.cuh"
#include "mfgb_internal.h"
#include "mfgb_launch.cuh"

namespace mfgb {
namespace {

// cells per CTA (about 7 warps of NQ^2-thread cells) and resident CTAs per SM:
// the shapes of the TwoSum BP3 kernel
template <int NQ> struct Bp3FxElems {
  static constexpr int value =
      NQ == 3 ? 24 : NQ == 4 ? 14 : NQ == 5 ? 9 : NQ == 6 ? 6 : NQ == 7 ? 4 : NQ <= 9 ? 2 : 1;
};
template <int NQ> struct Bp3FxMinBlocks { static constexpr int value = NQ <= 6 ? 2 : 1; };

// B (and D, when given) as float pairs with the bound factors of the offset
// accumulation: K = 2 (1 + 2^-20) times the row and column sums of |B|, |D|
template <int NM, int NQ>
void fill_basis(const double *hB, const double *hDG, BasisQFX<NM, NQ> &b) {
  const double K = 2.0 * (1.0 + std::ldexp(1.0, -20));
  for (int t = 0; t < NQ * NM; ++t) {
    b.Bh[t] = (float)hB[t];
    b.Bl[t] = (float)(hB[t] - (double)b.Bh[t]);
  }
  for (int t = 0; t < NQ * NQ; ++t) {
    b.Dh[t] = hDG ? (float)hDG[t] : 0.f;
    b.Dl[t] = hDG ? (float)(hDG[t] - (double)b.Dh[t]) : 0.f;
  }
  double LB = 0.0;
  for (int q = 0; q < NQ; ++q) {
    double rb = 0.0, rd = 0.0, cd = 0.0;
    for (int i = 0; i < NM; ++i) rb += std::fabs((double)b.Bh[q * NM + i]);
    for (int m = 0; m < NQ; ++m) {
      rd += std::fabs((double)b.Dh[q * NQ + m]);
      cd += std::fabs((double)b.Dh[m * NQ + q]);
    }
    b.rB[q] = (float)(K * rb);
    b.rD[q] = (float)(K * rd);
    b.cD[q] = (float)(K * cd);
    LB = std::max(LB, rb);
  }
  for (int i = 0; i < NM; ++i) {
    double cb = 0.0;
    for (int q = 0; q < NQ; ++q) cb += std::fabs((double)b.Bh[q * NM + i]);
    b.cB[i] = (float)(K * cb);
  }
  b.LB = (float)(LB * (1.0 + std::ldexp(1.0, -20)));
  b.K = (float)K;
}

template <int NM, int NQ, bool MT>
cudaError_t bp3fx_launch(int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                         const double *src, double *dst, const double *hB, const double *hDG,
                         cudaStream_t s, const int *done) {
  constexpr int E = Bp3FxElems<NQ>::value, MB = Bp3FxMinBlocks<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  constexpr size_t smem = TmaLayoutQ<NM, NQ, E, ArithDF, 4>::total;
  BasisQFX<NM, NQ> b;
  fill_basis(hB, hDG, b);
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bp3fx_tma_kernel<NM, NQ, E, MB, MT>, threads, smem));
  const int64_t batches = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * num_sms()));
  bp3fx_tma_kernel<NM, NQ, E, MB, MT><<<grid, threads, smem, s>>>(n_cells, map, G, gexp, src, dst,
                                                                    b, done, device_error_flag());
  return cudaGetLastError();
}

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
                   const double *hDG, cudaStream_t s, const int *done) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || (reinterpret_cast<uintptr_t>(Gfx) & 15u)) return cudaErrorInvalidValue;
  // bulk copies of the dof-map tiles need a 16-byte aligned map
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  const int extra = nq - degree - 1;  // 1: BP3 (q = p + 2), 0: Gauss p + 1
  if (extra != 0 && extra != 1) return cudaErrorInvalidValue;
  switch (degree * 2 + extra) {
#define MFGB_BP3FX(P, X)                                                                         \
  case 2 * P + X:                                                                                \
    return mt ? bp3fx_launch<P + 1, P + 1 + X, true>(n_cells, map, Gfx, gexp, src, dst, hB, hDG, s, \
                                                     done)                                        \
              : bp3fx_launch<P + 1, P + 1 + X, false>(n_cells, map, Gfx, gexp, src, dst, hB, hDG,  \
                                                      s, done);
    MFGB_BP3FX(1, 1) MFGB_BP3FX(2, 1) MFGB_BP3FX(3, 1) MFGB_BP3FX(4, 1) MFGB_BP3FX(5, 1)
    MFGB_BP3FX(6, 1) MFGB_BP3FX(7, 1) MFGB_BP3FX(8, 1)
    MFGB_BP3FX(1, 0) MFGB_BP3FX(2, 0) MFGB_BP3FX(3, 0) MFGB_BP3FX(4, 0) MFGB_BP3FX(5, 0)
    MFGB_BP3FX(6, 0) MFGB_BP3FX(7, 0) MFGB_BP3FX(8, 0)
#undef MFGB_BP3FX
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb
