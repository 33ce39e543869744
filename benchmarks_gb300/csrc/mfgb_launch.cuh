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

// bulk-TMA column kernel: elements per CTA, per arithmetic (default: as the
// column kernel)
template <int N, class A> struct ElemsPerCtaTma { static constexpr int value = ElemsPerCta<N>::value; };
template <> struct ElemsPerCtaTma<5, ArithF32> { static constexpr int value = 6; };
template <> struct ElemsPerCtaTma<5, ArithDF> { static constexpr int value = 5; };

// Alternative cells per CTA for the autotuner's shapes 3 (column) and 4 (bulk
// TMA): a CTA of (nearly) whole warps, smaller or larger than the default.  Their
// residency cap follows the register budget of the arithmetic (about 128
// registers a thread for FP64 and double-float, 64 for FP32).  Offered (value
// > 0) for FP32 at every N and for FP64 / double-float up to N = 5; above that
// a 128-register cap spills, and the alternative shapes run as shapes 0 / 2.
template <int N> struct AltElemsN;
template <> struct AltElemsN<2> { static constexpr int value = 16; };  // 64 threads
template <> struct AltElemsN<3> { static constexpr int value = 14; };  // 126
template <> struct AltElemsN<4> { static constexpr int value = 4; };   // 64
template <> struct AltElemsN<5> { static constexpr int value = 10; };  // 250
template <> struct AltElemsN<6> { static constexpr int value = 3; };   // 108
template <> struct AltElemsN<7> { static constexpr int value = 6; };   // 294
template <> struct AltElemsN<8> { static constexpr int value = 1; };   // 64
template <> struct AltElemsN<9> { static constexpr int value = 4; };   // 324
template <int N, class A> struct AltElems { static constexpr int value = 0; };
template <int N> struct AltElems<N, ArithF32> { static constexpr int value = AltElemsN<N>::value; };
template <int N> struct AltElems<N, ArithF64> {
  static constexpr int value = N <= 5 ? AltElemsN<N>::value : 0;
};
template <int N> struct AltElems<N, ArithDF> {
  static constexpr int value = N <= 5 ? AltElemsN<N>::value : 0;
};
template <class A> struct RegThreads { static constexpr int value = 512; };
template <> struct RegThreads<ArithF32> { static constexpr int value = 1024; };
template <int N, int E, class A> struct AltMinBlocks {
  static constexpr int threads = (E * N * N + 31) / 32 * 32;
  static constexpr int raw = RegThreads<A>::value / (threads > 0 ? threads : 1);
  static constexpr int value = raw < 1 ? 1 : (raw > 8 ? 8 : raw);
};

// point-per-thread kernel: elements per CTA (CTA = E * N^3 threads)
template <int N> struct ElemsPerCtaPt;
template <> struct ElemsPerCtaPt<2> { static constexpr int value = 32; };
template <> struct ElemsPerCtaPt<3> { static constexpr int value = 8; };
template <> struct ElemsPerCtaPt<4> { static constexpr int value = 4; };
template <> struct ElemsPerCtaPt<5> { static constexpr int value = 2; };
template <> struct ElemsPerCtaPt<6> { static constexpr int value = 2; };
template <> struct ElemsPerCtaPt<7> { static constexpr int value = 1; };
template <> struct ElemsPerCtaPt<8> { static constexpr int value = 1; };
template <> struct ElemsPerCtaPt<9> { static constexpr int value = 1; };

// Kernel shape: 0 = column (thread owns an i-column), 1 = point-per-thread,
// 2 = column with TMA-prefetched geometric factors.  Default per
// (arithmetic, N); overridable at run time (autotuner).
// 5 and 6 (double-float only, GLL operators): the offset-accumulation kernel of
// mfgb_bk5fx.cuh at the shape-2 and shape-4 cells per CTA; elsewhere they run as 2 / 4.
enum { SHAPE_COLUMN = 0, SHAPE_POINT = 1, SHAPE_TMA = 2, SHAPE_COLUMN_ALT = 3, SHAPE_TMA_ALT = 4,
       SHAPE_FX = 5, SHAPE_FX_ALT = 6 };
int kernel_shape(int arith_class, int N);  // mfgb_api.cu
int *device_error_flag();                  // mfgb_api.cu

template <class A> struct ArithClass { static constexpr int value = 0; };  // FP64
template <> struct ArithClass<ArithDF> { static constexpr int value = 1; };
template <> struct ArithClass<ArithDFG64> { static constexpr int value = 1; };
template <> struct ArithClass<ArithF32> { static constexpr int value = 2; };

inline int num_sms() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 152;
  }
  return sms;
}

// CTAs per SM of one kernel instantiation (queried once).  Sets the kernel's
// dynamic shared-memory limit to smem: without it, dynamic plus static shared
// memory above 48 KB fails at launch.
template <class K>
int ctas_per_sm(K kernel, int threads, size_t smem) {
  int ps = 0;
  if (smem > 0) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ps, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    ps = 0;
  }
  return ps;
}

// grid for a persistent launch: all resident CTAs, capped by the work
template <int N, class A, bool EVEC, bool EN>
int bk5_grid(int64_t n_cells, int shape) {
  static int per_sm[5] = {-1, -1, -1, -1, -1};
  int &ps = per_sm[shape];
  int E = 1;
  constexpr int EA = AltElems<N, A>::value;
  if (shape == SHAPE_COLUMN_ALT) {
    if constexpr (EA > 0 && !EVEC) {
      E = EA;
      if (ps < 0)
        ps = ctas_per_sm(bk5_kernel_mb<N, EA, A, EVEC, EN, AltMinBlocks<N, EA, A>::value>,
                         EA * N * N, 0);
    }
  } else if (shape == SHAPE_TMA_ALT) {
    if constexpr (EA > 0 && !EVEC) {
      E = EA;
      if (ps < 0)
        ps = ctas_per_sm(bk5_tma_kernel<N, EA, A, EN, AltMinBlocks<N, EA, A>::value>, EA * N * N,
                         TmaLayout<N, EA, A>::total);
    }
  } else if (shape == SHAPE_POINT) {
    E = ElemsPerCtaPt<N>::value;
    if (ps < 0) ps = ctas_per_sm(bk5_pt_kernel<N, ElemsPerCtaPt<N>::value, A, EVEC, EN>, E * N * N * N, 0);
  } else if (shape == SHAPE_TMA) {
    constexpr int ET = ElemsPerCtaTma<N, A>::value;
    E = ET;
    if (ps < 0)
      ps = ctas_per_sm(bk5_tma_kernel<N, ET, A, EN>, ET * N * N, TmaLayout<N, ET, A>::total);
  } else {
    E = ElemsPerCta<N>::value;
    if (ps < 0) {
      if constexpr (ColumnMinBlocks<N, A>::value > 0)
        ps = ctas_per_sm(bk5_kernel_capped<N, ElemsPerCta<N>::value, A, EVEC, EN>, E * N * N, 0);
      else
        ps = ctas_per_sm(bk5_kernel<N, ElemsPerCta<N>::value, A, EVEC, EN>, E * N * N, 0);
    }
  }
  if (ps < 1) ps = 1;
  const int64_t n_batches = (n_cells + E - 1) / E;
  const int64_t full = (int64_t)ps * num_sms();
  return (int)std::max<int64_t>(1, std::min<int64_t>(n_batches, full));
}

template <int N, class A, bool EVEC, bool EN>
cudaError_t bk5_launch(int64_t n_cells, const uint32_t *map, const typename A::GType *G,
                       const typename A::VecT *src, typename A::VecT *dst,
                       const Basis<N, A> &basis, double *partials, int *grid_used,
                       cudaStream_t stream, const int *done_flag = nullptr) {
  int shape = kernel_shape(ArithClass<A>::value, N);
  if (shape == SHAPE_FX) shape = SHAPE_TMA;
  if (shape == SHAPE_FX_ALT) shape = SHAPE_TMA_ALT;
  // without an alternative cells-per-CTA instantiation (E-vector mode, other
  // arithmetic, large N) shapes 3 / 4 run as 0 / 2; bulk copies need 16-byte
  // aligned tiles: caller arrays that are not 16-byte aligned use the column
  // kernel
  if (EVEC || AltElems<N, A>::value == 0) {
    if (shape == SHAPE_COLUMN_ALT) shape = SHAPE_COLUMN;
    if (shape == SHAPE_TMA_ALT) shape = SHAPE_TMA;
  }
  if ((shape == SHAPE_TMA || shape == SHAPE_TMA_ALT) &&
      (EVEC || ((reinterpret_cast<uintptr_t>(G) | reinterpret_cast<uintptr_t>(map)) & 15u)))
    shape = SHAPE_COLUMN;
  const int grid = bk5_grid<N, A, EVEC, EN>(n_cells, shape);
  if (grid_used) *grid_used = grid;
  if (n_cells <= 0) return cudaSuccess;
  constexpr int EA = AltElems<N, A>::value;
  constexpr int MBA = AltMinBlocks<N, EA, A>::value;
  if (shape == SHAPE_COLUMN_ALT) {
    if constexpr (EA > 0 && !EVEC)
      bk5_kernel_mb<N, EA, A, EVEC, EN, MBA><<<grid, EA * N * N, 0, stream>>>(
          n_cells, map, G, src, dst, basis, partials, done_flag);
  } else if (shape == SHAPE_TMA_ALT) {
    if constexpr (EA > 0 && !EVEC)
      bk5_tma_kernel<N, EA, A, EN, MBA><<<grid, EA * N * N, TmaLayout<N, EA, A>::total, stream>>>(
          n_cells, map, G, src, dst, basis, partials, done_flag, device_error_flag());
  } else if (shape == SHAPE_POINT) {
    constexpr int E = ElemsPerCtaPt<N>::value;
    bk5_pt_kernel<N, E, A, EVEC, EN><<<grid, E * N * N * N, 0, stream>>>(
        n_cells, map, G, src, dst, basis, partials, done_flag);
  } else if (shape == SHAPE_TMA) {
    if constexpr (!EVEC) {
      constexpr int E = ElemsPerCtaTma<N, A>::value;
      bk5_tma_kernel<N, E, A, EN><<<grid, E * N * N, TmaLayout<N, E, A>::total, stream>>>(
          n_cells, map, G, src, dst, basis, partials, done_flag, device_error_flag());
    }
  } else {
    constexpr int E = ElemsPerCta<N>::value;
    if constexpr (ColumnMinBlocks<N, A>::value > 0)
      bk5_kernel_capped<N, E, A, EVEC, EN><<<grid, E * N * N, 0, stream>>>(
          n_cells, map, G, src, dst, basis, partials, done_flag);
    else
      bk5_kernel<N, E, A, EVEC, EN><<<grid, E * N * N, 0, stream>>>(n_cells, map, G, src, dst,
                                                                     basis, partials, done_flag);
  }
  return cudaGetLastError();
}

}  // namespace mfgb
