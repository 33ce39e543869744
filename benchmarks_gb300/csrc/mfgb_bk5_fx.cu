// The FP64-accurate collocation operator with offset double-float accumulation
// (mfgb_bk5fx.cuh): its launcher, and the set-up of the per-cell scaled
// geometric factors it reads.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "mfgb_bk5fx.cuh"
#include "mfgb_internal.h"
#include "mfgb_launch.cuh"

namespace mfgb {

// cells per CTA and resident CTAs per SM of the two thread-block shapes
// (shape 4 = the alternative cells per CTA of mfgb_launch.cuh)
template <int N> struct FxElems { static constexpr int value = ElemsPerCtaTma<N, ArithDF>::value; };
template <int N> struct FxMinBlocks { static constexpr int value = TmaMinBlocks<N, ArithDF>::value; };
template <int N> struct FxAltElems { static constexpr int value = AltElemsN<N>::value; };
template <int N> struct FxAltMinBlocks {
  static constexpr int value = AltMinBlocks<N, FxAltElems<N>::value, ArithDF>::value;
};
// n = 7..9: fewer cells per CTA and more resident CTAs (registers from -Xptxas
// -v: n = 7, 2 cells, 3 CTAs: 158, no spill; n = 8, 1 cell, 4 CTAs: 179, no
// spill; n = 9, 2 cells, 2 CTAs: 168 with a 48-byte spill, 1 cell, 3 CTAs: 168
// with 32 bytes), where the wide cells of 1-CTA shapes left too few warps
template <> struct FxElems<7> { static constexpr int value = 2; };
template <> struct FxMinBlocks<7> { static constexpr int value = 3; };
template <> struct FxAltMinBlocks<8> { static constexpr int value = 4; };
template <> struct FxMinBlocks<9> { static constexpr int value = 2; };
template <> struct FxAltElems<9> { static constexpr int value = 1; };
template <> struct FxAltMinBlocks<9> { static constexpr int value = 3; };

// test hook: applications left whose first copy wait is made to run out
static std::atomic<int> g_expire{0};

static bool take_expire() {
  for (int c = g_expire.load(); c > 0; c = g_expire.load())
    if (g_expire.compare_exchange_weak(c, c - 1)) return true;
  return false;
}

template <int N, int E, int MB, bool MT>
static cudaError_t fx_launch(int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                             const double *src, double *dst, const BasisFX<N> &b, cudaStream_t s,
                             const int *done) {
  constexpr size_t smem = TmaLayout<N, E, ArithDF>::total;
  static int per_sm = -1;
  if (per_sm < 0)
    per_sm = std::max(1, ctas_per_sm(bk5fx_tma_kernel<N, E, MB, MT>, E * N * N, smem));
  const int64_t nb = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm * num_sms()));
  if (n_cells <= 0) return cudaSuccess;
  bk5fx_tma_kernel<N, E, MB, MT><<<grid, E * N * N, smem, s>>>(n_cells, map, G, gexp, src, dst, b,
                                                                done, device_error_flag());
  return cudaGetLastError();
}

// one application with the copy-wait test hook (the default cells per CTA)
template <int N>
static cudaError_t fx_launch_expire(int64_t n_cells, const uint32_t *map, const float2 *G,
                                    const int *gexp, const double *src, double *dst,
                                    const BasisFX<N> &b, cudaStream_t s, const int *done) {
  constexpr int E = FxElems<N>::value, MB = FxMinBlocks<N>::value;
  constexpr size_t smem = TmaLayout<N, E, ArithDF>::total;
  ctas_per_sm(bk5fx_tma_kernel<N, E, MB, false, true>, E * N * N, smem);  // sets the smem limit
  const int64_t nb = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)num_sms()));
  bk5fx_tma_kernel<N, E, MB, false, true><<<grid, E * N * N, smem, s>>>(
      n_cells, map, G, gexp, src, dst, b, done, device_error_flag());
  return cudaGetLastError();
}

template <int N>
static cudaError_t fx_with_basis(int64_t n_cells, const uint32_t *map, const float2 *G,
                                 const int *gexp, const double *src, double *dst, const double *D,
                                 cudaStream_t s, const int *done) {
  BasisFX<N> b;
  const double K = 2.0 * (1.0 + std::ldexp(1.0, -20));
  for (int q = 0; q < N * N; ++q) {
    b.Dh[q] = (float)D[q];
    b.Dl[q] = (float)(D[q] - (double)b.Dh[q]);
  }
  for (int i = 0; i < N; ++i) {
    double rs = 0.0, cs = 0.0;
    for (int m = 0; m < N; ++m) {
      rs += std::fabs((double)b.Dh[i * N + m]);
      cs += std::fabs((double)b.Dh[m * N + i]);
    }
    b.cg[i] = (float)(K * rs);
    b.ci[i] = (float)(K * cs);
  }
  b.K = (float)K;
  // bulk copies of the dof-map tiles need a 16-byte aligned map
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  const bool alt = kernel_shape(ArithClass<ArithDF>::value, N) == SHAPE_FX_ALT;
  constexpr int E = FxElems<N>::value, MB = FxMinBlocks<N>::value;
  constexpr int EA = FxAltElems<N>::value, MBA = FxAltMinBlocks<N>::value;
  if (take_expire()) return fx_launch_expire<N>(n_cells, map, G, gexp, src, dst, b, s, done);
  if (alt)
    return mt ? fx_launch<N, EA, MBA, true>(n_cells, map, G, gexp, src, dst, b, s, done)
              : fx_launch<N, EA, MBA, false>(n_cells, map, G, gexp, src, dst, b, s, done);
  return mt ? fx_launch<N, E, MB, true>(n_cells, map, G, gexp, src, dst, b, s, done)
            : fx_launch<N, E, MB, false>(n_cells, map, G, gexp, src, dst, b, s, done);
}

// the basis pairs and bound factors of the collocation kernels
template <int N>
static BasisFX<N> basis_fx(const double *D) {
  BasisFX<N> b;
  const double K = 2.0 * (1.0 + std::ldexp(1.0, -20));
  for (int q = 0; q < N * N; ++q) {
    b.Dh[q] = (float)D[q];
    b.Dl[q] = (float)(D[q] - (double)b.Dh[q]);
  }
  for (int i = 0; i < N; ++i) {
    double rs = 0.0, cs = 0.0;
    for (int m = 0; m < N; ++m) {
      rs += std::fabs((double)b.Dh[i * N + m]);
      cs += std::fabs((double)b.Dh[m * N + i]);
    }
    b.cg[i] = (float)(K * rs);
    b.ci[i] = (float)(K * cs);
  }
  b.K = (float)K;
  return b;
}

// the L-vector form on the caller's FP64 G (16-byte aligned)
template <int N, bool MT>
static cudaError_t fx_g64_launch(int64_t n_cells, const uint32_t *map, const double *G,
                                 const double *src, double *dst, const double *D,
                                 cudaStream_t s) {
  const BasisFX<N> b = basis_fx<N>(D);
  constexpr int E = FxElems<N>::value, MB = FxMinBlocks<N>::value;
  constexpr size_t smem = TmaLayout<N, E, ArithF64>::total;
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk5fx_g64_kernel<N, E, MB, MT>, E * N * N, smem));
  const int64_t nb = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm * num_sms()));
  bk5fx_g64_kernel<N, E, MB, MT><<<grid, E * N * N, smem, s>>>(n_cells, map, G, src, dst, b,
                                                                device_error_flag());
  return cudaGetLastError();
}

cudaError_t bk5_fx_g64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                       const double *src, double *dst, const double *D, cudaStream_t s) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || (reinterpret_cast<uintptr_t>(G) & 15u)) return cudaErrorInvalidValue;
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  switch (N) {
#define MFGB_FXG(NN)                                                      \
  case NN:                                                                \
    return mt ? fx_g64_launch<NN, true>(n_cells, map, G, src, dst, D, s) \
              : fx_g64_launch<NN, false>(n_cells, map, G, src, dst, D, s);
    MFGB_FXG(2) MFGB_FXG(3) MFGB_FXG(4) MFGB_FXG(5) MFGB_FXG(6) MFGB_FXG(7) MFGB_FXG(8) MFGB_FXG(9)
#undef MFGB_FXG
    default: return cudaErrorInvalidValue;
  }
}

// the E-vector form: FP64 G (16-byte aligned), contiguous input and output
template <int N>
static cudaError_t fx_evec_with_basis(int64_t nelmt, const double *G, const double *src,
                                      double *dst, const double *D, cudaStream_t s) {
  const BasisFX<N> b = basis_fx<N>(D);
  constexpr int E = FxElems<N>::value, MB = FxMinBlocks<N>::value;
  constexpr size_t smem = TmaLayout<N, E, ArithF64>::total;
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk5fx_evec_kernel<N, E, MB>, E * N * N, smem));
  const int64_t nb = (nelmt + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm * num_sms()));
  bk5fx_evec_kernel<N, E, MB><<<grid, E * N * N, smem, s>>>(nelmt, G, src, dst, b,
                                                            device_error_flag());
  return cudaGetLastError();
}

cudaError_t bk5_fx_evec(int N, int64_t nelmt, const double *G, const double *src, double *dst,
                        const double *D, cudaStream_t s) {
  if (nelmt <= 0) return cudaSuccess;
  if (reinterpret_cast<uintptr_t>(G) & 15u) return cudaErrorInvalidValue;  // bulk copies
  switch (N) {
#define MFGB_FXEV(NN) \
  case NN: return fx_evec_with_basis<NN>(nelmt, G, src, dst, D, s);
    MFGB_FXEV(2) MFGB_FXEV(3) MFGB_FXEV(4) MFGB_FXEV(5) MFGB_FXEV(6) MFGB_FXEV(7) MFGB_FXEV(8)
    MFGB_FXEV(9)
#undef MFGB_FXEV
    default: return cudaErrorInvalidValue;
  }
}

// the BK6 vector Laplacian: 3 interleaved components per DoF on one scaled G
template <int N, bool MT>
static cudaError_t fx_bk6_launch(int64_t n_cells, const uint32_t *map, const float2 *G,
                                 const int *gexp, const double *src, double *dst, const double *D,
                                 cudaStream_t s) {
  const BasisFX<N> b = basis_fx<N>(D);
  constexpr int E = FxElems<N>::value, MB = FxMinBlocks<N>::value;
  constexpr size_t smem = TmaLayout<N, E, ArithDF>::total;
  static int per_sm = -1;
  if (per_sm < 0)
    per_sm = std::max(1, ctas_per_sm(bk6fx_tma_kernel<N, E, MB, MT, 3>, E * N * N, smem));
  const int64_t nb = (n_cells + E - 1) / E;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm * num_sms()));
  bk6fx_tma_kernel<N, E, MB, MT, 3><<<grid, E * N * N, smem, s>>>(n_cells, map, G, gexp, src, dst,
                                                                  b, device_error_flag());
  return cudaGetLastError();
}

cudaError_t bk6_fx(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                   const double *src, double *dst, const double *D, cudaStream_t s) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || (reinterpret_cast<uintptr_t>(G) & 15u)) return cudaErrorInvalidValue;
  const bool mt = (reinterpret_cast<uintptr_t>(map) & 15u) == 0;
  switch (N) {
#define MFGB_FX6(NN)                                                              \
  case NN:                                                                        \
    return mt ? fx_bk6_launch<NN, true>(n_cells, map, G, gexp, src, dst, D, s) \
              : fx_bk6_launch<NN, false>(n_cells, map, G, gexp, src, dst, D, s);
    MFGB_FX6(2) MFGB_FX6(3) MFGB_FX6(4) MFGB_FX6(5) MFGB_FX6(6) MFGB_FX6(7) MFGB_FX6(8) MFGB_FX6(9)
#undef MFGB_FX6
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t bk5_fx(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                   const double *src, double *dst, const double *D, cudaStream_t s,
                   const int *done) {
  if (n_cells <= 0) return cudaSuccess;
  if (map == nullptr || (reinterpret_cast<uintptr_t>(G) & 15u)) return cudaErrorInvalidValue;
  switch (N) {
#define MFGB_FXCASE(NN) \
  case NN: return fx_with_basis<NN>(n_cells, map, G, gexp, src, dst, D, s, done);
    MFGB_FXCASE(2) MFGB_FXCASE(3) MFGB_FXCASE(4) MFGB_FXCASE(5) MFGB_FXCASE(6) MFGB_FXCASE(7)
    MFGB_FXCASE(8) MFGB_FXCASE(9)
#undef MFGB_FXCASE
    default: return cudaErrorInvalidValue;
  }
}

// Per-cell scaled split of the FP64 geometric factors: one warp per cell finds
// the largest biased exponent e among the cell's 6 n^3 values (and its per_j
// JxW values, when given) and writes them times 2^-(e - 1022) as float pairs
// (hi = nearest float, lo = nearest float of the remainder); gexp[cell] =
// e - 1022 (0 for an all-zero cell).  Values more than 2^126 below the cell's
// largest lose their low digits or flush to zero, far below the operator's
// accuracy bar relative to the cell's largest term.
__global__ void g_to_fx_kernel(int64_t n_cells, int per_cell, const double *__restrict__ G,
                               float2 *__restrict__ out, int *__restrict__ gexp, int per_j,
                               const double *__restrict__ J, float2 *__restrict__ jout) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  auto split = [](double x, int off) {
    const double y = scalbn(x, -off);
    const float hi = __double2float_rn(y);
    return make_float2(hi, __double2float_rn(y - (double)hi));
  };
  for (int64_t c = warp; c < n_cells; c += n_warps) {
    const double *g = G + c * per_cell;
    const double *j = J + c * per_j;
    int em = 0;
    for (int t = lane; t < per_cell; t += 32) {
      const int e = dexp(g[t]);
      em = max(em, e == 0x7FF ? 0 : e);
    }
    for (int t = lane; t < per_j; t += 32) {
      const int e = dexp(j[t]);
      em = max(em, e == 0x7FF ? 0 : e);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xFFFFFFFFu, em, o));
    const int off = fx_offset(em);
    for (int t = lane; t < per_cell; t += 32) out[c * per_cell + t] = split(g[t], off);
    for (int t = lane; t < per_j; t += 32) jout[c * per_j + t] = split(j[t], off);
    if (lane == 0) gexp[c] = off;
  }
}

cudaError_t g_to_fx(int64_t n_cells, int per_cell, const double *G, float2 *Gfx, int *gexp,
                    cudaStream_t s, int per_cell_j, const double *J, float2 *Jfx) {
  if (n_cells <= 0) return cudaSuccess;
  if (per_cell_j > 0 && (!J || !Jfx)) return cudaErrorInvalidValue;
  const int64_t blocks = std::min<int64_t>((n_cells + 7) / 8, 152 * 32);
  g_to_fx_kernel<<<(int)blocks, 256, 0, s>>>(n_cells, per_cell, G, Gfx, gexp,
                                             per_cell_j > 0 ? per_cell_j : 0, J, Jfx);
  return cudaGetLastError();
}

}  // namespace mfgb

extern "C" mfgb_status mfgb_test_expire_copy_wait(int n) {
  if (n < 0) {
    mfgb::set_error("mfgb_test_expire_copy_wait: n must be >= 0");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb::g_expire.store(n);
  return MFGB_OK;
}
