// mfgb_bp3fx_launch.cuh -- host side of the Gauss-point offset-accumulation
// kernel (mfgb_bp3fx.cuh): its thread-block shapes, the basis split with the
// bound factors, and the launcher, shared by the Laplacian and Helmholtz
// translation units.
#pragma once
#include <algorithm>
#include <cmath>

#include "mfgb_bp3fx.cuh"
#include "mfgb_launch.cuh"

namespace mfgb {

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
inline void fill_basis(const double *hB, const double *hDG, BasisQFX<NM, NQ> &b) {
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

template <int NM, int NQ, bool MT, bool MASS = false>
inline cudaError_t bp3fx_launch(int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                         const double *src, double *dst, const double *hB, const double *hDG,
                         cudaStream_t s, const int *done, const float2 *jxw) {
  constexpr int E = Bp3FxElems<NQ>::value, MB = Bp3FxMinBlocks<NQ>::value;
  constexpr int threads = E * NQ * NQ;
  constexpr size_t smem = TmaLayoutQ<NM, NQ, E, ArithDF, 4>::total;
  BasisQFX<NM, NQ> b;
  fill_basis(hB, hDG, b);
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bp3fx_tma_kernel<NM, NQ, E, MB, MT, MASS>, threads, smem));
  const int64_t batches = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(batches, (int64_t)per_sm * num_sms()));
  bp3fx_tma_kernel<NM, NQ, E, MB, MT, MASS><<<grid, threads, smem, s>>>(
      n_cells, map, G, gexp, src, dst, b, done, device_error_flag(), jxw);
  return cudaGetLastError();
}

}  // namespace mfgb
