// mfgb_dispatch.cuh -- runtime degree dispatch for the BK5 kernels.
#pragma once
#include <cmath>
#include <type_traits>

#include "mfgb_launch.cuh"

namespace mfgb {

template <class A> struct BasisValue;
template <> struct BasisValue<ArithF64> {
  static double from(double d) { return d; }
};
template <> struct BasisValue<ArithF32> {
  static float from(double d) { return (float)d; }
};
template <> struct BasisValue<ArithDF> {
  static df from(double d) {
    df r;
    r.hi = (float)d;
    r.lo = (float)(d - (double)r.hi);
    return r;
  }
};
template <> struct BasisValue<ArithDFG64> : BasisValue<ArithDF> {};

// Fills the even-odd tables of a basis and sets b.eo when D64 is the
// derivative of nodes symmetric about the cell centre (D[N-1-i][N-1-m] = -D[i][m]
// to rounding), for the plain arithmetics; caller-supplied matrices of the
// kernel seams need not have that symmetry and keep the dense form.
template <int N, class A>
void fill_even_odd(Basis<N, A> &b, const double *D64) {
  b.eo = 0;
  if constexpr (std::is_same<A, ArithF64>::value || std::is_same<A, ArithF32>::value) {
    double big = 0.0, asym = 0.0;
    for (int q = 0; q < N * N; ++q) big = std::max(big, std::fabs(D64[q]));
    for (int i = 0; i < N; ++i)
      for (int m = 0; m < N; ++m)
        asym = std::max(asym, std::fabs(D64[(N - 1 - i) * N + (N - 1 - m)] + D64[i * N + m]));
    if (asym > 1e-13 * big) return;
    constexpr int H = N / 2;
    for (int i = 0; i < (N + 1) / 2; ++i) {
      for (int m = 0; m < H; ++m) {
        b.Pg[i][m] = BasisValue<A>::from(0.5 * (D64[i * N + m] + D64[i * N + N - 1 - m]));
        b.Qg[i][m] = BasisValue<A>::from(0.5 * (D64[i * N + m] - D64[i * N + N - 1 - m]));
        b.Pt[i][m] = BasisValue<A>::from(0.5 * (D64[m * N + i] + D64[(N - 1 - m) * N + i]));
        b.Qt[i][m] = BasisValue<A>::from(0.5 * (D64[m * N + i] - D64[(N - 1 - m) * N + i]));
      }
      if (N % 2) {
        b.Pg[i][H] = BasisValue<A>::from(D64[i * N + H]);
        b.Pt[i][H] = BasisValue<A>::from(D64[H * N + i]);
      }
    }
    b.eo = 1;
  }
}

template <int N, class A, bool EVEC, bool EN>
cudaError_t bk5_with_basis(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                           const typename A::VecT *src, typename A::VecT *dst, const double *D64,
                           double *partials, int *grid, cudaStream_t s, const int *done) {
  Basis<N, A> b{};
  for (int q = 0; q < N * N; ++q) b.D[q] = BasisValue<A>::from(D64[q]);
  fill_even_odd(b, D64);
  return bk5_launch<N, A, EVEC, EN>(n_cells, map, G, src, dst, b, partials, grid, s, done);
}

template <class A, bool EVEC, bool EN>
cudaError_t bk5_dispatch(int N, int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                         const typename A::VecT *src, typename A::VecT *dst, const double *D64,
                         double *partials, int *grid, cudaStream_t s,
                         const int *done = nullptr) {
  switch (N) {
#define MFGB_CASE(NN) \
  case NN: return bk5_with_basis<NN, A, EVEC, EN>(n_cells, map, G, src, dst, D64, partials, grid, s, done);
    MFGB_CASE(2) MFGB_CASE(3) MFGB_CASE(4) MFGB_CASE(5) MFGB_CASE(6) MFGB_CASE(7) MFGB_CASE(8)
    MFGB_CASE(9)
#undef MFGB_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb

namespace mfgb {

// cells per CTA of the Gauss-point TMA kernel: whole warps at n = 5 (250
// threads), else as the column kernel
template <int N> struct GaussTmaElems { static constexpr int value = N == 5 ? 10 : ElemsPerCta<N>::value; };
// residency of the Gauss-point TMA kernel: the register budget of the
// arithmetic up to n = 5 (as AltMinBlocks), one CTA per SM's worth above
template <int N, int E, class A> struct GaussTmaMinBlocks {
  static constexpr int value = N <= 5 ? AltMinBlocks<N, E, A>::value : 1;
};

template <int N, class A, bool EN>
cudaError_t bk5g_with_basis(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                            const typename A::VecT *src, typename A::VecT *dst, const double *DG64,
                            const double *B64, double *partials, int *grid, cudaStream_t s,
                            const int *done, const typename A::GType *jxw) {
  constexpr int E = ElemsPerCta<N>::value;
  BasisG<N, A> b;
  for (int q = 0; q < N * N; ++q) {
    b.D[q] = BasisValue<A>::from(DG64[q]);
    b.B[q] = BasisValue<A>::from(B64[q]);
  }
  const int64_t n_batches = (n_cells + E - 1) / E;
  // L-vector mode with 16-byte aligned G and map: the bulk-TMA pipeline
  const bool tma = !EN && map != nullptr &&
                   ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(map)) & 15u) == 0;
  if (tma) {
    constexpr int ET = GaussTmaElems<N>::value;
    constexpr int MB = GaussTmaMinBlocks<N, ET, A>::value;
    constexpr size_t smem = TmaLayout<N, ET, A>::total;
    static int per_sm_tma = -1;
    if (per_sm_tma < 0)
      per_sm_tma = std::max(1, ctas_per_sm(bk5g_tma_kernel<N, ET, A, MB>, ET * N * N, smem));
    const int64_t nb = (n_cells + ET - 1) / ET;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm_tma * num_sms()));
    if (grid) *grid = g;
    if (n_cells <= 0) return cudaSuccess;
    bk5g_tma_kernel<N, ET, A, MB><<<g, ET * N * N, smem, s>>>(n_cells, map, G, src, dst, b, done,
                                                              jxw, device_error_flag());
    return cudaGetLastError();
  }
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk5g_kernel<N, E, A, EN>, E * N * N, 0));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(n_batches, (int64_t)per_sm * num_sms()));
  if (grid) *grid = g;
  if (n_cells <= 0) return cudaSuccess;
  bk5g_kernel<N, E, A, EN><<<g, E * N * N, 0, s>>>(n_cells, map, G, src, dst, b, partials, done,
                                                   jxw);
  return cudaGetLastError();
}

template <class A, bool EN>
cudaError_t bk5g_dispatch(int N, int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                          const typename A::VecT *src, typename A::VecT *dst, const double *DG,
                          const double *B, double *partials, int *grid, cudaStream_t s,
                          const int *done, const typename A::GType *jxw) {
  switch (N) {
#define MFGB_GCASE(NN) \
  case NN:             \
    return bk5g_with_basis<NN, A, EN>(n_cells, map, G, src, dst, DG, B, partials, grid, s, done, jxw);
    MFGB_GCASE(2) MFGB_GCASE(3) MFGB_GCASE(4) MFGB_GCASE(5) MFGB_GCASE(6) MFGB_GCASE(7)
    MFGB_GCASE(8) MFGB_GCASE(9)
#undef MFGB_GCASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb

namespace mfgb {

// cells per CTA of the BK6 TMA kernel: as the Gauss-point one
template <int N> struct Bk6TmaElems { static constexpr int value = GaussTmaElems<N>::value; };

template <int N, class A>
cudaError_t bk6_with_basis(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                           const typename A::VecT *src, typename A::VecT *dst, const double *D64,
                           cudaStream_t s) {
  constexpr int E = ElemsPerCta<N>::value;
  Basis<N, A> b{};
  for (int q = 0; q < N * N; ++q) b.D[q] = BasisValue<A>::from(D64[q]);
  const size_t smem = sizeof(typename A::GType) * E * 6 * N * N * N +
                      3 * sizeof(typename A::V) * E * N * N * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  // 16-byte aligned G and map: the bulk-TMA pipeline
  if (((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(map)) & 15u) == 0) {
    constexpr int ET = Bk6TmaElems<N>::value;
    constexpr int MB = GaussTmaMinBlocks<N, ET, A>::value;
    constexpr size_t smem_t = TmaLayout<N, ET, A>::total;
    static int per_sm_tma = -1;
    if (per_sm_tma < 0)
      per_sm_tma = std::max(1, ctas_per_sm(bk6_tma_kernel<N, ET, A, 3, MB>, ET * N * N, smem_t));
    const int64_t nb = (n_cells + ET - 1) / ET;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(nb, (int64_t)per_sm_tma * num_sms()));
    if (n_cells <= 0) return cudaSuccess;
    bk6_tma_kernel<N, ET, A, 3, MB><<<g, ET * N * N, smem_t, s>>>(n_cells, map, G, src, dst, b,
                                                                  device_error_flag());
    return cudaGetLastError();
  }
  static int per_sm = -1;
  if (per_sm < 0) per_sm = std::max(1, ctas_per_sm(bk6_kernel<N, E, A, 3>, E * N * N, smem));
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(n_batches, (int64_t)per_sm * num_sms()));
  if (n_cells <= 0) return cudaSuccess;
  bk6_kernel<N, E, A, 3><<<g, E * N * N, smem, s>>>(n_cells, map, G, src, dst, b);
  return cudaGetLastError();
}

template <class A>
cudaError_t bk6_dispatch(int N, int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                         const typename A::VecT *src, typename A::VecT *dst, const double *D,
                         cudaStream_t s) {
  switch (N) {
#define MFGB_VCASE(NN) case NN: return bk6_with_basis<NN, A>(n_cells, map, G, src, dst, D, s);
    MFGB_VCASE(2) MFGB_VCASE(3) MFGB_VCASE(4) MFGB_VCASE(5) MFGB_VCASE(6) MFGB_VCASE(7)
    MFGB_VCASE(8) MFGB_VCASE(9)
#undef MFGB_VCASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace mfgb
