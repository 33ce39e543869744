// mfgb_bk5.cuh -- fused BK5 operator kernels (gather -> D -> G -> D^T -> scatter).
//
// One CTA holds E elements; thread (e, j, k) owns the column i = 0..N-1 of
// element e in registers (the reference's 2D (j,k) thread map with i in
// registers, CEED_BK/include/kernels/BK5/templated_cuda_kernels.cuh:44-122).
// The r-direction contraction runs in registers with D entries as
// compile-time constant-bank operands; s and t go through shared memory.
//
// L-vector mode (map != nullptr) follows the reference's L-vector kernel
// (bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:129-151 gather with the
// 0xFFFFFFFF mask, :406-426 atomic scatter) in the GLL-collocated form
// (interpolation matrices are identities, so steps 2-4 and 9-11 of that kernel
// drop out).  E-vector mode (map == nullptr) reads in[e][l] and writes out[e][l].
//
// With WITH_ENERGY the kernel also returns, per CTA, sum_e u_e . (A_e u_e) in
// FP64 (the element-local form of p.Ap for conjugate gradients); CTAs visit
// their elements in a fixed order, so the partials are deterministic.
#pragma once
#include "mfgb_common.cuh"

namespace mfgb {

// Resident CTAs the compiler must fit per SM (register cap) for the column
// kernel; 0 leaves the register count to the compiler.  FP32 applies are
// memory-latency bound and at N = 5 the compiler's choice (67 registers)
// stops at about 40 % of the warp slots (measured: 11 % faster capped).
template <int N, class A> struct ColumnMinBlocks { static constexpr int value = 0; };
template <> struct ColumnMinBlocks<5, ArithF32> { static constexpr int value = 5; };

// even-odd form of the in-register contractions (plain arithmetics)
template <class A> struct EvenOddArith { static constexpr bool value = false; };
template <> struct EvenOddArith<ArithF64> { static constexpr bool value = true; };
template <> struct EvenOddArith<ArithF32> { static constexpr bool value = true; };

template <int N, int E, class A, bool EVEC, bool WITH_ENERGY>
__device__ __forceinline__ void bk5_column_body(const int64_t n_cells, const uint32_t *__restrict__ map,
               const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
               typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
               double *__restrict__ energy_partials, const int *__restrict__ done_flag) {
  if (done_flag != nullptr && *done_flag) return;  // solver already finished
  using V = typename A::V;
  using Acc = typename A::Acc;
  constexpr int N2 = N * N, N3 = N * N * N;
  constexpr bool kEvenOdd = EvenOddArith<A>::value;
  __shared__ V s_u[E * N3];
  __shared__ V s_vs[E * N3];
  __shared__ V s_vt[E * N3];

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;

  // rows / columns of D this thread needs with a runtime index
  V Dj[N], Dk[N], Dtj[N], Dtk[N];
#pragma unroll
  for (int m = 0; m < N; ++m) {
    Dj[m] = basis.D[j * N + m];
    Dk[m] = basis.D[k * N + m];
    Dtj[m] = basis.D[m * N + j];
    Dtk[m] = basis.D[m * N + k];
  }

  double energy = 0.0;
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    const int64_t cell = batch * E + el;
    const bool valid = cell < n_cells;
    V u[N];
    uint32_t idx[N];
    // ---- gather (with the Dirichlet mask)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      if (EVEC) {
        idx[i] = 0;
        u[i] = valid ? A::load_vec(src[cell * N3 + i * N2 + jk]) : A::zero_v();
      } else {
        idx[i] = valid ? __ldg(map + cell * N3 + i * N2 + jk) : MFGB_INVALID_DOF;
        u[i] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(__ldg(src + idx[i])) : A::zero_v();
      }
      s_u[el * N3 + i * N2 + jk] = u[i];
    }
    __syncthreads();

    // ---- reference gradient + metric apply; the r-derivative of the own
    // column first (even-odd form where the basis has it)
    V vr[N], qrv[N];
    if (kEvenOdd && basis.eo) {
      if constexpr (kEvenOdd) even_odd_apply<N, A>(basis.Pg, basis.Qg, u, qrv);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc ar;
        A::mul(ar, basis.D[i * N], u[0]);
#pragma unroll
        for (int m = 1; m < N; ++m) A::fma(ar, basis.D[i * N + m], u[m]);
        qrv[i] = A::finish(ar);
      }
    }
    const typename A::GType *Gc = G + (valid ? cell : 0) * 6 * N3 + jk;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc as, at;
      A::mul(as, Dj[0], s_u[el * N3 + i * N2 + k]);
      A::mul(at, Dk[0], s_u[el * N3 + i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(as, Dj[m], s_u[el * N3 + i * N2 + m * N + k]);
        A::fma(at, Dk[m], s_u[el * N3 + i * N2 + j * N + m]);
      }
      const V qr = qrv[i], qs = A::finish(as), qt = A::finish(at);
      const V grr = A::load_g(__ldg(Gc + 0 * N3 + i * N2));
      const V grs = A::load_g(__ldg(Gc + 1 * N3 + i * N2));
      const V grt = A::load_g(__ldg(Gc + 2 * N3 + i * N2));
      const V gss = A::load_g(__ldg(Gc + 3 * N3 + i * N2));
      const V gst = A::load_g(__ldg(Gc + 4 * N3 + i * N2));
      const V gtt = A::load_g(__ldg(Gc + 5 * N3 + i * N2));
      Acc br, bs, bt;
      A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      vr[i] = A::finish(br);
      s_vs[el * N3 + i * N2 + jk] = A::finish(bs);
      s_vt[el * N3 + i * N2 + jk] = A::finish(bt);
    }
    __syncthreads();

    // ---- integrate (D^T, sum of the three directions) + scatter; the
    // r-part from the own column first (even-odd form where available)
    V rv[N];
    if (kEvenOdd && basis.eo) {
      if constexpr (kEvenOdd) even_odd_apply<N, A>(basis.Pt, basis.Qt, vr, rv);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc a;
        A::mul(a, basis.D[i], vr[0]);
#pragma unroll
        for (int m = 1; m < N; ++m) A::fma(a, basis.D[m * N + i], vr[m]);
        rv[i] = A::finish(a);
      }
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::set(a, rv[i]);
#pragma unroll
      for (int m = 0; m < N; ++m) {
        A::fma(a, Dtj[m], s_vs[el * N3 + i * N2 + m * N + k]);
        A::fma(a, Dtk[m], s_vt[el * N3 + i * N2 + j * N + m]);
      }
      const V y = A::finish(a);
      if (EVEC) {
        if (valid) dst[cell * N3 + i * N2 + jk] = A::store_vec(y);
      } else if (idx[i] != MFGB_INVALID_DOF) {
        const typename A::VecT yv = A::store_vec(y);
        atomicAdd(dst + idx[i], yv);
        if (WITH_ENERGY) energy = __fma_rn((double)__ldg(src + idx[i]), (double)yv, energy);
      }
    }
    __syncthreads();
  }

  if (WITH_ENERGY) {
    // deterministic block reduction of the per-thread energies
    __shared__ double s_red[E * N * N];
    s_red[tid] = energy;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int t = 0; t < E * N * N; ++t) s += s_red[t];
      energy_partials[blockIdx.x] = s;
    }
  }
}

template <int N, int E, class A, bool EVEC, bool WITH_ENERGY>
__global__ void __launch_bounds__(E * N * N)
    bk5_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
               const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
               typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
               double *__restrict__ energy_partials, const int *__restrict__ done_flag) {
  bk5_column_body<N, E, A, EVEC, WITH_ENERGY>(n_cells, map, G, src, dst, basis, energy_partials,
                                              done_flag);
}

// the same with an explicit residency (register cap) of MB CTAs per SM
template <int N, int E, class A, bool EVEC, bool WITH_ENERGY, int MB>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5_kernel_mb(const int64_t n_cells, const uint32_t *__restrict__ map,
                  const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                  typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
                  double *__restrict__ energy_partials, const int *__restrict__ done_flag) {
  bk5_column_body<N, E, A, EVEC, WITH_ENERGY>(n_cells, map, G, src, dst, basis, energy_partials,
                                              done_flag);
}

// the same with the register cap of ColumnMinBlocks
template <int N, int E, class A, bool EVEC, bool WITH_ENERGY>
__global__ void __launch_bounds__(E * N * N, (ColumnMinBlocks<N, A>::value > 0
                                                  ? ColumnMinBlocks<N, A>::value : 1))
    bk5_kernel_capped(const int64_t n_cells, const uint32_t *__restrict__ map,
                      const typename A::GType *__restrict__ G,
                      const typename A::VecT *__restrict__ src, typename A::VecT *__restrict__ dst,
                      const Basis<N, A> basis, double *__restrict__ energy_partials,
                      const int *__restrict__ done_flag) {
  bk5_column_body<N, E, A, EVEC, WITH_ENERGY>(n_cells, map, G, src, dst, basis, energy_partials,
                                              done_flag);
}

}  // namespace mfgb

namespace mfgb {

// Point-per-thread variant: thread (e, i, j, k) owns one quadrature point of
// element e.  Registers stay low (the element tiles live in shared memory), so
// many more warps are resident to hide the gather / G latency; used for the
// double-float arithmetic whose FP32-pipe work per point is large.
template <int N, int E, class A, bool EVEC, bool WITH_ENERGY>
__global__ void __launch_bounds__(E * N * N * N)
    bk5_pt_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                  const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                  typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
                  double *__restrict__ energy_partials, const int *__restrict__ done_flag) {
  if (done_flag != nullptr && *done_flag) return;  // solver already finished
  using V = typename A::V;
  using Acc = typename A::Acc;
  constexpr int N2 = N * N, N3 = N * N * N;
  __shared__ V s_D[N2];
  __shared__ V s_u[E * N3];
  __shared__ V s_vr[E * N3];
  __shared__ V s_vs[E * N3];
  __shared__ V s_vt[E * N3];

  const int tid = threadIdx.x;
  const int el = tid / N3;
  const int q = tid - el * N3;
  const int i = q / N2;
  const int j = (q / N) % N;
  const int k = q % N;
  for (int t = tid; t < N2; t += blockDim.x) s_D[t] = basis.D[t];
  const V *su = s_u + el * N3;
  const V *svr = s_vr + el * N3;
  const V *svs = s_vs + el * N3;
  const V *svt = s_vt + el * N3;

  double energy = 0.0;
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    const int64_t cell = batch * E + el;
    const bool valid = cell < n_cells;
    uint32_t idx = MFGB_INVALID_DOF;
    typename A::VecT raw = 0;
    if (EVEC) {
      if (valid) raw = src[cell * N3 + q];
    } else {
      idx = valid ? __ldg(map + cell * N3 + q) : MFGB_INVALID_DOF;
      if (idx != MFGB_INVALID_DOF) raw = __ldg(src + idx);
    }
    // geometric factors of this point (issued early, consumed after the gradient)
    const typename A::GType *Gc = G + (valid ? cell : 0) * 6 * N3 + q;
    const typename A::GType g0 = __ldg(Gc + 0 * N3), g1 = __ldg(Gc + 1 * N3),
                            g2 = __ldg(Gc + 2 * N3), g3 = __ldg(Gc + 3 * N3),
                            g4 = __ldg(Gc + 4 * N3), g5 = __ldg(Gc + 5 * N3);
    s_u[tid] = A::load_vec(raw);
    __syncthreads();

    Acc ar, as, at;
    A::mul(ar, s_D[i * N], su[j * N + k]);
    A::mul(as, s_D[j * N], su[i * N2 + k]);
    A::mul(at, s_D[k * N], su[i * N2 + j * N]);
#pragma unroll
    for (int m = 1; m < N; ++m) {
      A::fma(ar, s_D[i * N + m], su[m * N2 + j * N + k]);
      A::fma(as, s_D[j * N + m], su[i * N2 + m * N + k]);
      A::fma(at, s_D[k * N + m], su[i * N2 + j * N + m]);
    }
    const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
    const V grr = A::load_g(g0), grs = A::load_g(g1), grt = A::load_g(g2);
    const V gss = A::load_g(g3), gst = A::load_g(g4), gtt = A::load_g(g5);
    Acc br, bs, bt;
    A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
    A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
    A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
    s_vr[tid] = A::finish(br);
    s_vs[tid] = A::finish(bs);
    s_vt[tid] = A::finish(bt);
    __syncthreads();

    Acc cr, cs, ct;
    A::mul(cr, s_D[i], svr[j * N + k]);
    A::mul(cs, s_D[j], svs[i * N2 + k]);
    A::mul(ct, s_D[k], svt[i * N2 + j * N]);
#pragma unroll
    for (int m = 1; m < N; ++m) {
      A::fma(cr, s_D[m * N + i], svr[m * N2 + j * N + k]);
      A::fma(cs, s_D[m * N + j], svs[i * N2 + m * N + k]);
      A::fma(ct, s_D[m * N + k], svt[i * N2 + j * N + m]);
    }
    A::merge(cr, cs);  // y = cr + cs + ct
    A::merge(cr, ct);
    const V y = A::finish(cr);
    if (EVEC) {
      if (valid) dst[cell * N3 + q] = A::store_vec(y);
    } else if (idx != MFGB_INVALID_DOF) {
      const typename A::VecT yv = A::store_vec(y);
      atomicAdd(dst + idx, yv);
      if (WITH_ENERGY) energy = __fma_rn((double)raw, (double)yv, energy);
    }
    __syncthreads();  // s_u / s_v* are rewritten by the next batch
  }

  if (WITH_ENERGY) {
    __shared__ double s_red[E * N3];
    s_red[tid] = energy;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int t = 0; t < E * N3; ++t) s += s_red[t];
      energy_partials[blockIdx.x] = s;
    }
  }
}

}  // namespace mfgb

#include "mfgb_tma.cuh"

namespace mfgb {

// Shared-memory layout of a bulk-TMA kernel's batch of E cells: G tile (6
// components at NQ^3 points per cell), dof-map tile (NM^3 per cell), NW work
// arrays of NQ^3 values per cell, two mbarriers.
template <int NM, int NQ, int E, class A, int NW = 3>
struct TmaLayoutQ {
  static constexpr int M3 = NM * NM * NM, Q3 = NQ * NQ * NQ;
  static constexpr size_t g_bytes = sizeof(typename A::GType) * E * 6 * Q3;
  static constexpr size_t map_bytes = ((size_t)E * M3 * 4 + 15) / 16 * 16;
  static constexpr size_t work_bytes = NW * sizeof(typename A::V) * E * Q3;
  static constexpr size_t total = g_bytes + map_bytes + work_bytes + 16;
  // tiles start at batch * (full tile): bulk copies only when every full tile
  // is a 16-byte multiple (then every batch's start is 16-byte aligned)
  static constexpr bool map_tma = (E * M3 * 4) % 16 == 0;
  static constexpr bool g_tma = g_bytes % 16 == 0;
};
template <int N, int E, class A> using TmaLayout = TmaLayoutQ<N, N, E, A>;

// One CTA's bulk-TMA staging of a batch's G tile and dof-map tile into shared
// memory, each completing on its own mbarrier; used by the collocation, the
// Gauss-point and the BP3 kernels.  issue_* run on one thread and complete the
// mbarrier phase whether or not a copy is issued.
template <int NM, int NQ, int E, class A>
struct TmaTilesQ {
  using GT = typename A::GType;
  using VT = typename A::VecT;
  using L = TmaLayoutQ<NM, NQ, E, A>;
  static constexpr int M2 = NM * NM, M3 = NM * NM * NM, Q3 = NQ * NQ * NQ;
  int64_t n_cells;
  const uint32_t *__restrict__ map;
  const GT *__restrict__ G;
  const VT *__restrict__ src;
  GT *sG;
  uint32_t *sMap;
  uint64_t *mbar_g, *mbar_m;
  bool map_ok = true;  // false: the map array is not 16-byte aligned (plain loads)

  __device__ __forceinline__ int cells_of(int64_t b) const {
    return (int)min((int64_t)E, n_cells - b * E);
  }
  __device__ __forceinline__ bool map_by_tma(int cells) const {
    return map_ok && L::map_tma && ((cells * M3 * 4) % 16 == 0);
  }
  // a bulk copy needs a 16-byte aligned start and a 16-byte multiple: 4-byte G
  // tiles of an odd number of cells with odd NQ^3 (an odd E, or the last batch)
  // are loaded by plain loads (load_g_plain)
  __device__ __forceinline__ bool g_by_tma(int cells) const {
    return L::g_tma && (sizeof(GT) * cells * 6 * Q3) % 16 == 0;
  }
  __device__ __forceinline__ void issue_g(int64_t b) const {
    const int cells = cells_of(b);
    const uint32_t gb = g_by_tma(cells) ? (uint32_t)(sizeof(GT) * cells * 6 * Q3) : 0u;
    mbar_arrive_expect_tx(mbar_g, gb);
    if (gb) bulk_g2s(sG, G + b * E * 6 * Q3, gb, mbar_g);
  }
  __device__ __forceinline__ void issue_map(int64_t b) const {
    const int cells = cells_of(b);
    const uint32_t mb = map_by_tma(cells) ? (uint32_t)(cells * M3 * 4) : 0u;
    mbar_arrive_expect_tx(mbar_m, mb);
    if (mb) bulk_g2s(sMap, map + b * E * M3, mb, mbar_m);
  }
  // after the G wait: the tile of a batch that had no bulk copy, by plain loads
  // (to be ordered before its readers by a barrier)
  __device__ __forceinline__ void load_g_plain(int64_t b, int tid, int nthreads) const {
    if (g_by_tma(cells_of(b))) return;
    const int64_t nG = (int64_t)cells_of(b) * 6 * Q3;
    const GT *Gb = G + b * E * 6 * Q3;
    for (int64_t t = tid; t < nG; t += nthreads) sG[t] = __ldg(Gb + t);
  }
  // node column (el, jk), jk = j * NM + k, of batch b: dof indices (from the
  // map tile or global) and the raw source values, into registers; threads
  // without a column (has_col false) get invalid indices
  __device__ __forceinline__ void gather(int64_t b, int el, int jk, uint32_t *idx, VT *raw,
                                         bool has_col = true) const {
    const int cells = cells_of(b);
    const bool valid = has_col && el < cells;
    const bool mt = map_by_tma(cells);
#pragma unroll
    for (int i = 0; i < NM; ++i) {
      idx[i] = valid ? (mt ? sMap[el * M3 + i * M2 + jk] : __ldg(map + (b * E + el) * M3 + i * M2 + jk))
                     : MFGB_INVALID_DOF;
      raw[i] = idx[i] != MFGB_INVALID_DOF ? __ldg(src + idx[i]) : VT(0);
    }
  }
};
template <int N, int E, class A> using TmaTiles = TmaTilesQ<N, N, E, A>;

// Column kernel with bulk-TMA prefetch.  Per batch b of E cells:
//   barrier A   wait for G(b) (mbarrier 0); the u(b) gather was prefetched
//               into registers during batch b-1
//   write s_u, barrier B, then TMA of map(b+next) (mbarrier 1)
//   gradient + metric (reads s_u, G(b) from shared memory), barrier C,
//   then TMA of G(b+next)
//   wait for map(b+next), prefetch u(b+next) = src[map] into registers,
//   integrate + atomic scatter of batch b
// Shared memory holds one G tile, one map tile and the three work arrays.
// err_flag (may be null) records a TMA wait that exceeded its time limit.
template <int N, class A> struct TmaMinBlocks { static constexpr int value = N <= 6 ? 2 : 1; };
// FP32 at N = 4, 5: the compiler's 86 / 107 registers leave 2-3 CTAs per SM
// (N = 5 runs 6 cells per CTA, ElemsPerCtaTma: 0.62 -> 0.54 ms at 2.95e7 DoFs).
// Double-float at N = 5 runs 5 cells per CTA (125 threads, 4 CTAs per SM by
// registers and shared memory): 3.76 -> 3.06 ms at 67.6M DoFs.
template <> struct TmaMinBlocks<4, ArithF32> { static constexpr int value = 4; };
template <> struct TmaMinBlocks<5, ArithF32> { static constexpr int value = 6; };
template <> struct TmaMinBlocks<5, ArithDF> { static constexpr int value = 4; };

template <int N, int E, class A, bool WITH_ENERGY, int MB = TmaMinBlocks<N, A>::value>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                   const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                   typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
                   double *__restrict__ energy_partials, const int *__restrict__ done_flag,
                   int *__restrict__ err_flag) {
  if (done_flag != nullptr && *done_flag) return;
  using V = typename A::V;
  using Acc = typename A::Acc;
  using GT = typename A::GType;
  using VT = typename A::VecT;
  using L = TmaLayout<N, E, A>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  GT *sG = reinterpret_cast<GT *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  V *s_u = reinterpret_cast<V *>(smem + L::g_bytes + L::map_bytes);
  V *s_vs = s_u + E * N3;
  V *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  V Dj[N], Dk[N], Dtj[N], Dtk[N];
#pragma unroll
  for (int m = 0; m < N; ++m) {
    Dj[m] = basis.D[j * N + m];
    Dk[m] = basis.D[k * N + m];
    Dtj[m] = basis.D[m * N + j];
    Dtk[m] = basis.D[m * N + k];
  }

  const TmaTiles<N, E, A> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm);
  };

  if (tid == 0) {
    mbar_init(mbar_g, 1);
    mbar_init(mbar_m, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    T.issue_g(batch);
    T.issue_map(batch);
  }
  uint32_t ph_g = 0, ph_m = 0;
  uint32_t idx[N];
  VT raw[N];
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw);
  }
  double energy = 0.0;

  for (; batch < n_batches; batch += gridDim.x) {
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase by barrier B
    V u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(raw[i]) : A::zero_v();
      s_u[el * N3 + i * N2 + jk] = u[i];
    }
    __syncthreads();  // barrier B: s_u ready; the map tile is free
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }

    const bool valid = el < T.cells_of(batch);
    V vr[N];
    const GT *Gc = sG + el * 6 * N3 + jk;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc ar, as, at;
      A::mul(ar, basis.D[i * N], u[0]);
      A::mul(as, Dj[0], s_u[el * N3 + i * N2 + k]);
      A::mul(at, Dk[0], s_u[el * N3 + i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(ar, basis.D[i * N + m], u[m]);
        A::fma(as, Dj[m], s_u[el * N3 + i * N2 + m * N + k]);
        A::fma(at, Dk[m], s_u[el * N3 + i * N2 + j * N + m]);
      }
      const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
      V grr = A::zero_v(), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = A::load_g(Gc[0 * N3 + i * N2]);
        grs = A::load_g(Gc[1 * N3 + i * N2]);
        grt = A::load_g(Gc[2 * N3 + i * N2]);
        gss = A::load_g(Gc[3 * N3 + i * N2]);
        gst = A::load_g(Gc[4 * N3 + i * N2]);
        gtt = A::load_g(Gc[5 * N3 + i * N2]);
      }
      Acc br, bs, bt;
      A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      vr[i] = A::finish(br);
      s_vs[el * N3 + i * N2 + jk] = A::finish(bs);
      s_vt[el * N3 + i * N2 + jk] = A::finish(bt);
    }
    __syncthreads();  // barrier C: G tile consumed, s_vs / s_vt ready
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }

    // this batch's scatter targets; then prefetch the next batch's gather
    uint32_t cur[N];
    VT cur_raw[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      cur[i] = idx[i];
      cur_raw[i] = raw[i];
    }
    if (has_next) {
      const bool okm = mbar_wait(mbar_m, ph_m);
      if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
      ph_m ^= 1u;
      if (okm) T.gather(next, el, jk, idx, raw);
      else
        for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = VT(0); }
    }

#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.D[i], vr[0]);
      A::fma(a, Dtj[0], s_vs[el * N3 + i * N2 + k]);
      A::fma(a, Dtk[0], s_vt[el * N3 + i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(a, basis.D[m * N + i], vr[m]);
        A::fma(a, Dtj[m], s_vs[el * N3 + i * N2 + m * N + k]);
        A::fma(a, Dtk[m], s_vt[el * N3 + i * N2 + j * N + m]);
      }
      const V y = A::finish(a);
      if (cur[i] != MFGB_INVALID_DOF) {
        const VT yv = A::store_vec(y);
        atomicAdd(dst + cur[i], yv);
        if (WITH_ENERGY) energy = __fma_rn((double)cur_raw[i], (double)yv, energy);
      }
    }
  }

  if (WITH_ENERGY) {
    __syncthreads();
    double *s_red = reinterpret_cast<double *>(s_u);  // work arrays are free now
    s_red[tid] = energy;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int t = 0; t < E * N * N; ++t) s += s_red[t];
      energy_partials[blockIdx.x] = s;
    }
  }
}

}  // namespace mfgb

namespace mfgb {

// Gauss-quadrature form (BP5 variant, nq = p + 1 Gauss points per direction):
// the deal.II-kernel form of the reference's L-vector kernel
// (bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:156-228 interpolate to
// the Gauss points, :230-302 collocation gradient + metric, :305-334 transpose,
// :340-404 interpolate back, :406-426 scatter).  Column layout as bk5_kernel;
// basis.D is the collocation derivative on the Gauss points, B the GLL basis
// at the Gauss points, B[q*N + i] = l_i(g_q).
template <int N, class A>
struct BasisG {
  typename A::V D[N * N];
  typename A::V B[N * N];
};

template <int N, int E, class A, bool WITH_ENERGY>
__global__ void __launch_bounds__(E * N * N)
    bk5g_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                typename A::VecT *__restrict__ dst, const BasisG<N, A> basis,
                double *__restrict__ energy_partials, const int *__restrict__ done_flag,
                const typename A::GType *__restrict__ jxw) {
  if (done_flag != nullptr && *done_flag) return;
  using V = typename A::V;
  using Acc = typename A::Acc;
  using VT = typename A::VecT;
  constexpr int N2 = N * N, N3 = N * N * N;
  __shared__ V s_a[E * N3];
  __shared__ V s_b[E * N3];
  __shared__ V s_c[E * N3];

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  V Dj[N], Dk[N], Dtj[N], Dtk[N];
#pragma unroll
  for (int m = 0; m < N; ++m) {
    Dj[m] = basis.D[j * N + m];
    Dk[m] = basis.D[k * N + m];
    Dtj[m] = basis.D[m * N + j];
    Dtk[m] = basis.D[m * N + k];
  }
  V *sa = s_a + el * N3, *sb = s_b + el * N3, *sc = s_c + el * N3;
  double energy = 0.0;
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    const int64_t cell = batch * E + el;
    const bool valid = cell < n_cells;
    uint32_t idx[N];
    VT raw[N];
    V u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      idx[i] = valid ? __ldg(map + cell * N3 + i * N2 + jk) : MFGB_INVALID_DOF;
      raw[i] = idx[i] != MFGB_INVALID_DOF ? __ldg(src + idx[i]) : VT(0);
      u[i] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(raw[i]) : A::zero_v();
      sa[i * N2 + jk] = u[i];
    }
    __syncthreads();
    // ---- interpolate to the Gauss points: along k, j (shared), i (registers)
    V t[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[k * N], sa[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[k * N + m], sa[i * N2 + j * N + m]);
      t[i] = A::finish(a);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) sb[i * N2 + jk] = t[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[j * N], sb[i * N2 + k]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[j * N + m], sb[i * N2 + m * N + k]);
      t[i] = A::finish(a);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[i * N], t[0]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[i * N + m], t[m]);
      u[i] = A::finish(a);
      sa[i * N2 + jk] = u[i];
    }
    __syncthreads();
    // ---- collocation gradient at the Gauss points + metric
    V vr[N];
    const typename A::GType *Gc = G + (valid ? cell : 0) * 6 * N3 + jk;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc ar, as, at;
      A::mul(ar, basis.D[i * N], u[0]);
      A::mul(as, Dj[0], sa[i * N2 + k]);
      A::mul(at, Dk[0], sa[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(ar, basis.D[i * N + m], u[m]);
        A::fma(as, Dj[m], sa[i * N2 + m * N + k]);
        A::fma(at, Dk[m], sa[i * N2 + j * N + m]);
      }
      const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
      const V grr = A::load_g(__ldg(Gc + 0 * N3 + i * N2));
      const V grs = A::load_g(__ldg(Gc + 1 * N3 + i * N2));
      const V grt = A::load_g(__ldg(Gc + 2 * N3 + i * N2));
      const V gss = A::load_g(__ldg(Gc + 3 * N3 + i * N2));
      const V gst = A::load_g(__ldg(Gc + 4 * N3 + i * N2));
      const V gtt = A::load_g(__ldg(Gc + 5 * N3 + i * N2));
      Acc br, bs, bt;
      A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      vr[i] = A::finish(br);
      sb[i * N2 + jk] = A::finish(bs);
      sc[i * N2 + jk] = A::finish(bt);
    }
    __syncthreads();
    // ---- transpose gradient (+ JxW u for the mass term), then back to the GLL
    // nodes along i (registers)
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.D[i], vr[0]);
      A::fma(a, Dtj[0], sb[i * N2 + k]);
      A::fma(a, Dtk[0], sc[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(a, basis.D[m * N + i], vr[m]);
        A::fma(a, Dtj[m], sb[i * N2 + m * N + k]);
        A::fma(a, Dtk[m], sc[i * N2 + j * N + m]);
      }
      if (jxw != nullptr && valid) A::fma(a, A::load_g(__ldg(jxw + cell * N3 + i * N2 + jk)), u[i]);
      t[i] = A::finish(a);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[i], t[0]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[m * N + i], t[m]);
      u[i] = A::finish(a);
    }
    __syncthreads();  // sb / sc consumed
#pragma unroll
    for (int i = 0; i < N; ++i) sa[i * N2 + jk] = u[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[j], sa[i * N2 + k]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[m * N + j], sa[i * N2 + m * N + k]);
      sb[i * N2 + jk] = A::finish(a);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[k], sb[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[m * N + k], sb[i * N2 + j * N + m]);
      const V y = A::finish(a);
      if (idx[i] != MFGB_INVALID_DOF) {
        const VT yv = A::store_vec(y);
        atomicAdd(dst + idx[i], yv);
        if (WITH_ENERGY) energy = __fma_rn((double)raw[i], (double)yv, energy);
      }
    }
    __syncthreads();
  }
  if (WITH_ENERGY) {
    double *s_red = reinterpret_cast<double *>(s_a);
    s_red[tid] = energy;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int t2 = 0; t2 < E * N * N; ++t2) s += s_red[t2];
      energy_partials[blockIdx.x] = s;
    }
  }
}

}  // namespace mfgb

namespace mfgb {

// The Gauss-point form with the bulk-TMA pipeline of bk5_tma_kernel: the next
// batch's G and dof-map tiles stream into shared memory while this batch is
// computed, and the next batch's gather is prefetched into registers during
// the integrate phase.  Per batch of E cells (W0, W1, W2 the work arrays):
//   A  wait G(b); W0 = u (prefetched gather); B; TMA map(b+next)
//      W1 = B_k W0; barrier; u = B_i B_j W1 (registers), W0 = u; barrier
//      gradient + metric (W0, G tile) -> vr (registers), W1, W2
//   C  TMA G(b+next); wait map(b+next), prefetch u(b+next)
//      integrate (+ JxW u for the mass term), back along i (registers); W0 = that
//      barrier; W1 = B_j^T W0; barrier; dst += B_k^T W1 (atomic)
// A JxW array (mass term) is read with plain loads.  Waits are bounded as in
// bk5_tma_kernel.
template <int N, int E, class A, int MB>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5g_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                    const typename A::GType *__restrict__ G,
                    const typename A::VecT *__restrict__ src, typename A::VecT *__restrict__ dst,
                    const BasisG<N, A> basis, const int *__restrict__ done_flag,
                    const typename A::GType *__restrict__ jxw, int *__restrict__ err_flag) {
  if (done_flag != nullptr && *done_flag) return;
  using V = typename A::V;
  using Acc = typename A::Acc;
  using GT = typename A::GType;
  using VT = typename A::VecT;
  using L = TmaLayout<N, E, A>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  GT *sG = reinterpret_cast<GT *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  V *w0 = reinterpret_cast<V *>(smem + L::g_bytes + L::map_bytes);
  V *w1 = w0 + E * N3;
  V *w2 = w1 + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA
  V *a0 = w0 + el * N3, *a1 = w1 + el * N3, *a2 = w2 + el * N3;
  // B and D in shared memory: each phase loads the rows / columns its thread
  // needs (indexed by j or k) into registers; rows indexed by the unrolled i
  // stay constant-bank operands
  __shared__ V sB[N * N], sD[N * N];
  for (int q = tid; q < N * N; q += blockDim.x) {
    sB[q] = basis.B[q];
    sD[q] = basis.D[q];
  }
  auto row = [&](const V *M, int r, V *out) {
#pragma unroll
    for (int m = 0; m < N; ++m) out[m] = M[r * N + m];
  };
  auto col = [&](const V *M, int c, V *out) {
#pragma unroll
    for (int m = 0; m < N; ++m) out[m] = M[m * N + c];
  };

  const TmaTiles<N, E, A> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm);
  };
  if (tid == 0) {
    mbar_init(mbar_g, 1);
    mbar_init(mbar_m, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    T.issue_g(batch);
    T.issue_map(batch);
  }
  uint32_t ph_g = 0, ph_m = 0;
  uint32_t idx[N];
  VT raw[N];
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw);
  }

  for (; batch < n_batches; batch += gridDim.x) {
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase
    const bool valid = el < T.cells_of(batch);
    const int64_t cell = batch * E + el;
#pragma unroll
    for (int i = 0; i < N; ++i)
      a0[i * N2 + jk] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(raw[i]) : A::zero_v();
    __syncthreads();  // barrier B: W0 ready; the map tile is free
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }
    // ---- interpolate to the Gauss points: along k (W0 -> W1), then j and i
    V t[N], u[N], c0[N], c1[N];
    row(sB, k, c0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, c0[0], a0[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, c0[m], a0[i * N2 + j * N + m]);
      a1[i * N2 + jk] = A::finish(a);
    }
    __syncthreads();
    row(sB, j, c0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, c0[0], a1[i * N2 + k]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, c0[m], a1[i * N2 + m * N + k]);
      t[i] = A::finish(a);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[i * N], t[0]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[i * N + m], t[m]);
      u[i] = A::finish(a);
      a0[i * N2 + jk] = u[i];
    }
    __syncthreads();
    // ---- collocation gradient at the Gauss points + metric (G tile in shared)
    V vr[N];
    const GT *Gc = sG + el * 6 * N3 + jk;
    row(sD, j, c0);
    row(sD, k, c1);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc ar, as, at;
      A::mul(ar, basis.D[i * N], u[0]);
      A::mul(as, c0[0], a0[i * N2 + k]);
      A::mul(at, c1[0], a0[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(ar, basis.D[i * N + m], u[m]);
        A::fma(as, c0[m], a0[i * N2 + m * N + k]);
        A::fma(at, c1[m], a0[i * N2 + j * N + m]);
      }
      const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
      V grr = A::zero_v(), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = A::load_g(Gc[0 * N3 + i * N2]);
        grs = A::load_g(Gc[1 * N3 + i * N2]);
        grt = A::load_g(Gc[2 * N3 + i * N2]);
        gss = A::load_g(Gc[3 * N3 + i * N2]);
        gst = A::load_g(Gc[4 * N3 + i * N2]);
        gtt = A::load_g(Gc[5 * N3 + i * N2]);
      }
      Acc br, bs, bt;
      A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      vr[i] = A::finish(br);
      a1[i * N2 + jk] = A::finish(bs);
      a2[i * N2 + jk] = A::finish(bt);
    }
    __syncthreads();  // barrier C: G tile consumed, W1 / W2 ready
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }
    // this batch's scatter targets; then prefetch the next batch's gather
    uint32_t cur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cur[i] = idx[i];
    if (has_next) {
      const bool okm = mbar_wait(mbar_m, ph_m);
      if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
      ph_m ^= 1u;
      if (okm) T.gather(next, el, jk, idx, raw);
      else
        for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = VT(0); }
    }
    // ---- transpose gradient (+ JxW u), then back to the GLL nodes along i
    col(sD, j, c0);
    col(sD, k, c1);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.D[i], vr[0]);
      A::fma(a, c0[0], a1[i * N2 + k]);
      A::fma(a, c1[0], a2[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        A::fma(a, basis.D[m * N + i], vr[m]);
        A::fma(a, c0[m], a1[i * N2 + m * N + k]);
        A::fma(a, c1[m], a2[i * N2 + j * N + m]);
      }
      if (jxw != nullptr && valid) A::fma(a, A::load_g(__ldg(jxw + cell * N3 + i * N2 + jk)), u[i]);
      t[i] = A::finish(a);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, basis.B[i], t[0]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, basis.B[m * N + i], t[m]);
      u[i] = A::finish(a);
    }
    // W0's last readers (the gradient) finished before barrier C
#pragma unroll
    for (int i = 0; i < N; ++i) a0[i * N2 + jk] = u[i];
    __syncthreads();  // W0 ready; W1 / W2 consumed
    col(sB, j, c0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, c0[0], a0[i * N2 + k]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, c0[m], a0[i * N2 + m * N + k]);
      a1[i * N2 + jk] = A::finish(a);
    }
    __syncthreads();
    col(sB, k, c0);
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::mul(a, c0[0], a1[i * N2 + j * N]);
#pragma unroll
      for (int m = 1; m < N; ++m) A::fma(a, c0[m], a1[i * N2 + j * N + m]);
      if (cur[i] != MFGB_INVALID_DOF) atomicAdd(dst + cur[i], A::store_vec(A::finish(a)));
    }
    // W1 is read above until barrier A of the next batch; W0 is rewritten only after it
  }
}

// BK6: the vector Laplacian with NC interleaved components (vec[NC*dof + c]),
// every component through the same scalar operator.  A batch's G tile is
// staged in shared memory once and used for all NC components, so the metric
// bytes are shared; dof map indices stay in registers across components.
template <int N, int E, class A, int NC>
__global__ void __launch_bounds__(E * N * N)
    bk6_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
               const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
               typename A::VecT *__restrict__ dst, const Basis<N, A> basis) {
  using V = typename A::V;
  using Acc = typename A::Acc;
  using GT = typename A::GType;
  using VT = typename A::VecT;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(16) unsigned char smem6[];
  GT *sG = reinterpret_cast<GT *>(smem6);
  V *s_u = reinterpret_cast<V *>(smem6 + sizeof(GT) * E * 6 * N3);
  V *s_vs = s_u + E * N3;
  V *s_vt = s_vs + E * N3;
  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  V Dj[N], Dk[N], Dtj[N], Dtk[N];
#pragma unroll
  for (int m = 0; m < N; ++m) {
    Dj[m] = basis.D[j * N + m];
    Dk[m] = basis.D[k * N + m];
    Dtj[m] = basis.D[m * N + j];
    Dtk[m] = basis.D[m * N + k];
  }
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    const int64_t c0 = batch * E;
    const int cells = (int)min((int64_t)E, n_cells - c0);
    const bool valid = el < cells;
    const int64_t cell = c0 + el;
    // stage this batch's G tile (coalesced, read once for all components)
    const GT *Gb = G + c0 * 6 * N3;
    for (int t = tid; t < cells * 6 * N3; t += blockDim.x) sG[t] = __ldg(Gb + t);
    uint32_t idx[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
      idx[i] = valid ? __ldg(map + cell * N3 + i * N2 + jk) : MFGB_INVALID_DOF;
#pragma unroll 1
    for (int c = 0; c < NC; ++c) {
      V u[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        u[i] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(__ldg(src + (size_t)NC * idx[i] + c))
                                          : A::zero_v();
        s_u[el * N3 + i * N2 + jk] = u[i];
      }
      __syncthreads();
      V vr[N];
      const GT *Gc = sG + el * 6 * N3 + jk;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc ar, as, at;
        A::mul(ar, basis.D[i * N], u[0]);
        A::mul(as, Dj[0], s_u[el * N3 + i * N2 + k]);
        A::mul(at, Dk[0], s_u[el * N3 + i * N2 + j * N]);
#pragma unroll
        for (int m = 1; m < N; ++m) {
          A::fma(ar, basis.D[i * N + m], u[m]);
          A::fma(as, Dj[m], s_u[el * N3 + i * N2 + m * N + k]);
          A::fma(at, Dk[m], s_u[el * N3 + i * N2 + j * N + m]);
        }
        const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
        V grr = A::zero_v(), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
        if (valid) {
          grr = A::load_g(Gc[0 * N3 + i * N2]);
          grs = A::load_g(Gc[1 * N3 + i * N2]);
          grt = A::load_g(Gc[2 * N3 + i * N2]);
          gss = A::load_g(Gc[3 * N3 + i * N2]);
          gst = A::load_g(Gc[4 * N3 + i * N2]);
          gtt = A::load_g(Gc[5 * N3 + i * N2]);
        }
        Acc br, bs, bt;
        A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
        A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
        A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
        vr[i] = A::finish(br);
        s_vs[el * N3 + i * N2 + jk] = A::finish(bs);
        s_vt[el * N3 + i * N2 + jk] = A::finish(bt);
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc a;
        A::mul(a, basis.D[i], vr[0]);
        A::fma(a, Dtj[0], s_vs[el * N3 + i * N2 + k]);
        A::fma(a, Dtk[0], s_vt[el * N3 + i * N2 + j * N]);
#pragma unroll
        for (int m = 1; m < N; ++m) {
          A::fma(a, basis.D[m * N + i], vr[m]);
          A::fma(a, Dtj[m], s_vs[el * N3 + i * N2 + m * N + k]);
          A::fma(a, Dtk[m], s_vt[el * N3 + i * N2 + j * N + m]);
        }
        const V y = A::finish(a);
        if (idx[i] != MFGB_INVALID_DOF) atomicAdd(dst + (size_t)NC * idx[i] + c, A::store_vec(y));
      }
      __syncthreads();
    }
  }
}


// BK6 with the bulk-TMA pipeline of bk5_tma_kernel: a batch's G tile (shared by
// the NC components) and the next batch's map tile arrive by bulk copies, and
// each component's gather is prefetched into registers during the integrate
// phase of the previous component (the next batch's first component during the
// last one).  Per batch of E cells:
//   A  wait G(b)
//   for each component c:
//        s_u = u_c (prefetched); B (c = 0: TMA map(b+next))
//        gradient + metric -> vr, s_vs, s_vt; C (last c: TMA G(b+next))
//        prefetch u_{c+1} (or, for the last c, wait map(b+next) and gather its u_0)
//        integrate + atomic scatter of component c
// Every wait is bounded (a timeout sets err_flag and the CTA returns).
template <int N, int E, class A, int NC, int MB>
__global__ void __launch_bounds__(E * N * N, MB)
    bk6_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                   const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                   typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
                   int *__restrict__ err_flag) {
  using V = typename A::V;
  using Acc = typename A::Acc;
  using GT = typename A::GType;
  using VT = typename A::VecT;
  using L = TmaLayout<N, E, A>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  GT *sG = reinterpret_cast<GT *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  V *s_u = reinterpret_cast<V *>(smem + L::g_bytes + L::map_bytes);
  V *s_vs = s_u + E * N3;
  V *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  V Dj[N], Dk[N], Dtj[N], Dtk[N];
#pragma unroll
  for (int m = 0; m < N; ++m) {
    Dj[m] = basis.D[j * N + m];
    Dk[m] = basis.D[k * N + m];
    Dtj[m] = basis.D[m * N + j];
    Dtk[m] = basis.D[m * N + k];
  }
  const TmaTiles<N, E, A> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  // dof indices of column (el, jk) of batch b, from the map tile or global
  auto indices = [&](int64_t b, uint32_t *idx) {
    const int cells = T.cells_of(b);
    const bool valid = el < cells;
    const bool mt = T.map_by_tma(cells);
#pragma unroll
    for (int i = 0; i < N; ++i)
      idx[i] = valid ? (mt ? sMap[el * N3 + i * N2 + jk] : __ldg(map + (b * E + el) * N3 + i * N2 + jk))
                     : MFGB_INVALID_DOF;
  };
  auto gather = [&](const uint32_t *idx, int c, VT *raw) {
#pragma unroll
    for (int i = 0; i < N; ++i)
      raw[i] = idx[i] != MFGB_INVALID_DOF ? __ldg(src + (size_t)NC * idx[i] + c) : VT(0);
  };
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm);
  };

  if (tid == 0) {
    mbar_init(mbar_g, 1);
    mbar_init(mbar_m, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    T.issue_g(batch);
    T.issue_map(batch);
  }
  uint32_t ph_g = 0, ph_m = 0;
  uint32_t idx[N], nidx[N];
  VT raw[N];
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    indices(batch, idx);
    gather(idx, 0, raw);
  }

  for (; batch < n_batches; batch += gridDim.x) {
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase by barrier B
    const bool valid = el < T.cells_of(batch);
    const GT *Gc = sG + el * 6 * N3 + jk;
#pragma unroll 1
    for (int c = 0; c < NC; ++c) {
      V u[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        u[i] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(raw[i]) : A::zero_v();
        s_u[el * N3 + i * N2 + jk] = u[i];
      }
      __syncthreads();  // barrier B: s_u ready (c = 0: the map tile is free)
      if (c == 0 && tid == 0 && has_next) {
        fence_proxy_async_smem();
        T.issue_map(next);
      }
      V vr[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc ar, as, at;
        A::mul(ar, basis.D[i * N], u[0]);
        A::mul(as, Dj[0], s_u[el * N3 + i * N2 + k]);
        A::mul(at, Dk[0], s_u[el * N3 + i * N2 + j * N]);
#pragma unroll
        for (int m = 1; m < N; ++m) {
          A::fma(ar, basis.D[i * N + m], u[m]);
          A::fma(as, Dj[m], s_u[el * N3 + i * N2 + m * N + k]);
          A::fma(at, Dk[m], s_u[el * N3 + i * N2 + j * N + m]);
        }
        const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
        V grr = A::zero_v(), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
        if (valid) {
          grr = A::load_g(Gc[0 * N3 + i * N2]);
          grs = A::load_g(Gc[1 * N3 + i * N2]);
          grt = A::load_g(Gc[2 * N3 + i * N2]);
          gss = A::load_g(Gc[3 * N3 + i * N2]);
          gst = A::load_g(Gc[4 * N3 + i * N2]);
          gtt = A::load_g(Gc[5 * N3 + i * N2]);
        }
        Acc br, bs, bt;
        A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
        A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
        A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
        vr[i] = A::finish(br);
        s_vs[el * N3 + i * N2 + jk] = A::finish(bs);
        s_vt[el * N3 + i * N2 + jk] = A::finish(bt);
      }
      __syncthreads();  // barrier C: s_vs / s_vt ready (last c: the G tile is consumed)
      if (c == NC - 1 && tid == 0 && has_next) {
        fence_proxy_async_smem();
        T.issue_g(next);
      }
      // prefetch the next component (or the next batch's first one)
      uint32_t cur[N];
#pragma unroll
      for (int i = 0; i < N; ++i) cur[i] = idx[i];
      if (c + 1 < NC) {
        gather(idx, c + 1, raw);
      } else if (has_next) {
        const bool okm = mbar_wait(mbar_m, ph_m);
        if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
        ph_m ^= 1u;
        if (okm) {
          indices(next, nidx);
#pragma unroll
          for (int i = 0; i < N; ++i) idx[i] = nidx[i];
          gather(idx, 0, raw);
        } else {
          for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = VT(0); }
        }
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Acc a;
        A::mul(a, basis.D[i], vr[0]);
        A::fma(a, Dtj[0], s_vs[el * N3 + i * N2 + k]);
        A::fma(a, Dtk[0], s_vt[el * N3 + i * N2 + j * N]);
#pragma unroll
        for (int m = 1; m < N; ++m) {
          A::fma(a, basis.D[m * N + i], vr[m]);
          A::fma(a, Dtj[m], s_vs[el * N3 + i * N2 + m * N + k]);
          A::fma(a, Dtk[m], s_vt[el * N3 + i * N2 + j * N + m]);
        }
        if (cur[i] != MFGB_INVALID_DOF)
          atomicAdd(dst + (size_t)NC * cur[i] + c, A::store_vec(A::finish(a)));
      }
    }
  }
}

}  // namespace mfgb
