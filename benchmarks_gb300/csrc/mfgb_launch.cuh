// mfgb_launch.cuh -- host-side launch helpers for the BK5 kernels.
#pragma once
#include <algorithm>
#include "mfgb_bk5.cuh"

namespace mfgb {

// elements per CTA for each N = p + 1 (CTA = E * N^2 threads)
template <int N> struct ElemsPerCta;
template <> struct ElemsPerCta<2> { static constexpr int value = 32; };
template <> struct ElemsPerCta<3> { static constexpr int value = 16; };
template <> struct ElemsPerCta<4> { static constexpr int value = 8; };
template <> struct ElemsPerCta<5> { static constexpr int value = 8; };
template <> struct ElemsPerCta<6> { static constexpr int value = 4; };
template <> struct ElemsPerCta<7> { static constexpr int value = 4; };
template <> struct ElemsPerCta<8> { static constexpr int value = 2; };
template <> struct ElemsPerCta<9> { static constexpr int value = 2; };

inline int num_sms() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
  }
  return sms;
}

// grid for a persistent launch: all resident CTAs, capped by the work
template <int N, class A, bool EVEC, bool EN>
int bk5_grid(int64_t n_cells) {
  constexpr int E = ElemsPerCta<N>::value;
  static int per_sm = -1;
  if (per_sm < 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bk5_kernel<N, E, A, EVEC, EN>,
                                                      E * N * N, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
  }
  const int64_t n_batches = (n_cells + E - 1) / E;
  const int64_t full = (int64_t)per_sm * num_sms();
  return (int)std::max<int64_t>(1, std::min<int64_t>(n_batches, full));
}

template <int N, class A, bool EVEC, bool EN>
cudaError_t bk5_launch(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                       const typename A::VecT *src, typename A::VecT *dst,
                       const Basis<N, A> &basis, double *partials, int *grid_used,
                       cudaStream_t stream, const int *done_flag = nullptr) {
  constexpr int E = ElemsPerCta<N>::value;
  const int grid = bk5_grid<N, A, EVEC, EN>(n_cells);
  if (grid_used) *grid_used = grid;
  if (n_cells <= 0) return cudaSuccess;
  bk5_kernel<N, E, A, EVEC, EN><<<grid, E * N * N, 0, stream>>>(n_cells, map, G, src, dst, basis,
                                                                 partials, done_flag);
  return cudaGetLastError();
}

}  // namespace mfgb
