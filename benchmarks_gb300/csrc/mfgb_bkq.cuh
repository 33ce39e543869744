// mfgb_bkq.cuh -- CEED BK1 (mass) and BK3 (Laplacian) E-vector operators:
// NM = p + 1 modes per direction interpolated to NQ quadrature points
// (NQ = p + 2 in the CEED definition), sum factorised.
//
//   BK1: out_e = B^T (JxW_e o (B x B x B) in_e)
//        (CEED_BK/include/kernels/BK1/serial_kernels.hpp:20-121)
//   BK3: out_e = B^T (D^T G_e D) (B x B x B) in_e, D the collocation derivative
//        at the NQ points (CEED_BK/include/kernels/BK3/serial_kernels.hpp:29-188)
//
// Layouts (point and mode indices with direction 0 slowest, like BK5):
// basis[q*NM + i], dbasis[q*NQ + m], JxW[e][NQ^3], G[e][6][NQ^3] (rr rs rt ss st
// tt; the reference CUDA BK3 kernel's layout, templated_cuda_kernels.cuh:156-161),
// in/out[e][NM^3].  With a dof map (L-vector mode, the BP3 operator) the input
// is gathered through map[e][NM^3] and the output scatter-added atomically.
//
// GB300 structure (bkq_kernel): a CTA holds E elements, NQ^2 threads per
// element.  The interpolation passes run one 1D line per thread through shared
// memory; the Laplacian's gradient/metric/integrate phase uses the BK5 column
// layout (thread (q, r) keeps the direction-0 column of its points in
// registers).  Arithmetic is FP64 or double-float (policy A).  The BP3 L-vector
// operator has its own kernel with the bulk-TMA pipeline (bp3_tma_kernel, below);
// bkq_kernel serves the E-vector seams and unaligned BP3 slabs.
#pragma once
#include "mfgb_bk5.cuh"

namespace mfgb {

template <int NQ> struct BkqElems { static constexpr int value = NQ <= 3 ? 16 : NQ <= 5 ? 8 : NQ <= 7 ? 4 : NQ <= 8 ? 2 : 1; };

template <int NM, int NQ, class A, bool LAPLACE>
__global__ void __launch_bounds__(NQ * NQ * BkqElems<NQ>::value)
    bkq_kernel(const int64_t nelmt, const double *__restrict__ basis,
               const double *__restrict__ dbasis, const double *__restrict__ coef,
               const double *__restrict__ in, double *__restrict__ out,
               const uint32_t *__restrict__ map) {
  using V = typename A::V;
  using Acc = typename A::Acc;
  constexpr int E = BkqElems<NQ>::value;
  constexpr int NQ2 = NQ * NQ, NQ3 = NQ2 * NQ, NM2 = NM * NM, NM3 = NM2 * NM;
  __shared__ V sB[NQ * NM];
  __shared__ V sD[LAPLACE ? NQ * NQ : 1];
  __shared__ V s0[E * NQ3];
  __shared__ V s1[E * NQ3];
  __shared__ V s2[LAPLACE ? E * NQ3 : 1];
  __shared__ V s3[LAPLACE ? E * NQ3 : 1];

  const int tid = threadIdx.x;
  const int el = tid / NQ2;
  const int lt = tid - el * NQ2;
  for (int i = tid; i < NQ * NM; i += blockDim.x) sB[i] = A::load_vec(basis[i]);
  if (LAPLACE)
    for (int i = tid; i < NQ * NQ; i += blockDim.x) sD[i] = A::load_vec(dbasis[i]);
  __syncthreads();
  V *a0 = s0 + el * NQ3, *a1 = s1 + el * NQ3;

  const int64_t n_batches = (nelmt + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    const int64_t e = batch * E + el;
    const bool valid = e < nelmt;
    // E-vector: in[e][NM^3]; L-vector (map != nullptr): gather through the map
    for (int t = lt; t < NM3; t += NQ2) {
      if (!valid) {
        a0[t] = A::zero_v();
      } else if (map) {
        const uint32_t d = __ldg(map + e * NM3 + t);
        a0[t] = d != MFGB_INVALID_DOF ? A::load_vec(__ldg(in + d)) : A::zero_v();
      } else {
        a0[t] = A::load_vec(in[e * NM3 + t]);
      }
    }
    __syncthreads();
    // ---- interpolate: direction 0 (i -> p), lines (j, k)
    for (int t = lt; t < NM2; t += NQ2) {
      V r[NM];
#pragma unroll
      for (int i = 0; i < NM; ++i) r[i] = a0[i * NM2 + t];
#pragma unroll
      for (int p = 0; p < NQ; ++p) {
        Acc a;
        A::mul(a, sB[p * NM], r[0]);
#pragma unroll
        for (int i = 1; i < NM; ++i) A::fma(a, sB[p * NM + i], r[i]);
        a1[p * NM2 + t] = A::finish(a);
      }
    }
    __syncthreads();
    // direction 1 (j -> q), lines (p, k): a1[p][j][k] -> a0[p][q][k]
    for (int t = lt; t < NQ * NM; t += NQ2) {
      const int p = t / NM, k = t - p * NM;
      V r[NM];
#pragma unroll
      for (int j = 0; j < NM; ++j) r[j] = a1[p * NM2 + j * NM + k];
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        Acc a;
        A::mul(a, sB[q * NM], r[0]);
#pragma unroll
        for (int j = 1; j < NM; ++j) A::fma(a, sB[q * NM + j], r[j]);
        a0[(p * NQ + q) * NM + k] = A::finish(a);
      }
    }
    __syncthreads();
    // direction 2 (k -> r), lines (p, q) = lt: a0[p][q][k] -> a1[p][q][r]
    {
      V r[NM];
#pragma unroll
      for (int k = 0; k < NM; ++k) r[k] = a0[lt * NM + k];
#pragma unroll
      for (int rr = 0; rr < NQ; ++rr) {
        Acc a;
        A::mul(a, sB[rr * NM], r[0]);
#pragma unroll
        for (int k = 1; k < NM; ++k) A::fma(a, sB[rr * NM + k], r[k]);
        V v = A::finish(a);
        if (!LAPLACE) {  // mass: JxW at the point
          Acc m;
          A::zero(m);
          A::fma(m, valid ? A::load_vec(__ldg(coef + e * NQ3 + lt * NQ + rr)) : A::zero_v(), v);
          v = A::finish(m);
        }
        a1[lt * NQ + rr] = v;
      }
    }
    __syncthreads();
    if constexpr (LAPLACE) {
      // ---- collocation gradient + metric; thread (q, r) = lt owns the p-column
      V *a2 = s2 + el * NQ3, *a3 = s3 + el * NQ3;
      const int q = lt / NQ, r = lt - q * NQ;
      V u[NQ], vr[NQ];
#pragma unroll
      for (int p = 0; p < NQ; ++p) u[p] = a1[p * NQ2 + lt];
      const double *Ge = coef + (valid ? e : 0) * 6 * NQ3 + lt;
#pragma unroll
      for (int p = 0; p < NQ; ++p) {
        Acc ar, as, at;
        A::mul(ar, sD[p * NQ], u[0]);
        A::mul(as, sD[q * NQ], a1[p * NQ2 + r]);
        A::mul(at, sD[r * NQ], a1[p * NQ2 + q * NQ]);
#pragma unroll
        for (int m = 1; m < NQ; ++m) {
          A::fma(ar, sD[p * NQ + m], u[m]);
          A::fma(as, sD[q * NQ + m], a1[p * NQ2 + m * NQ + r]);
          A::fma(at, sD[r * NQ + m], a1[p * NQ2 + q * NQ + m]);
        }
        const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
        const V grr = A::load_vec(__ldg(Ge + 0 * NQ3 + p * NQ2));
        const V grs = A::load_vec(__ldg(Ge + 1 * NQ3 + p * NQ2));
        const V grt = A::load_vec(__ldg(Ge + 2 * NQ3 + p * NQ2));
        const V gss = A::load_vec(__ldg(Ge + 3 * NQ3 + p * NQ2));
        const V gst = A::load_vec(__ldg(Ge + 4 * NQ3 + p * NQ2));
        const V gtt = A::load_vec(__ldg(Ge + 5 * NQ3 + p * NQ2));
        Acc br, bs, bt;
        A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
        A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
        A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
        vr[p] = A::finish(br);
        a2[p * NQ2 + lt] = A::finish(bs);
        a3[p * NQ2 + lt] = A::finish(bt);
      }
      __syncthreads();  // a1 is no longer read: it receives the integrated values
#pragma unroll
      for (int p = 0; p < NQ; ++p) {
        Acc a;
        A::mul(a, sD[p], vr[0]);
        A::fma(a, sD[q], a2[p * NQ2 + r]);
        A::fma(a, sD[r], a3[p * NQ2 + q * NQ]);
#pragma unroll
        for (int m = 1; m < NQ; ++m) {
          A::fma(a, sD[m * NQ + p], vr[m]);
          A::fma(a, sD[m * NQ + q], a2[p * NQ2 + m * NQ + r]);
          A::fma(a, sD[m * NQ + r], a3[p * NQ2 + q * NQ + m]);
        }
        a1[p * NQ2 + lt] = A::finish(a);
      }
      __syncthreads();
    }
    // ---- transposed interpolation: direction 2 (r -> k), lines (p, q) = lt
    {
      V r[NQ];
#pragma unroll
      for (int rr = 0; rr < NQ; ++rr) r[rr] = a1[lt * NQ + rr];
#pragma unroll
      for (int k = 0; k < NM; ++k) {
        Acc a;
        A::mul(a, sB[k], r[0]);
#pragma unroll
        for (int rr = 1; rr < NQ; ++rr) A::fma(a, sB[rr * NM + k], r[rr]);
        a0[lt * NM + k] = A::finish(a);
      }
    }
    __syncthreads();
    // direction 1 (q -> j), lines (p, k): a0[p][q][k] -> a1[p][j][k]
    for (int t = lt; t < NQ * NM; t += NQ2) {
      const int p = t / NM, k = t - p * NM;
      V r[NQ];
#pragma unroll
      for (int q = 0; q < NQ; ++q) r[q] = a0[(p * NQ + q) * NM + k];
#pragma unroll
      for (int j = 0; j < NM; ++j) {
        Acc a;
        A::mul(a, sB[j], r[0]);
#pragma unroll
        for (int q = 1; q < NQ; ++q) A::fma(a, sB[q * NM + j], r[q]);
        a1[p * NM2 + j * NM + k] = A::finish(a);
      }
    }
    __syncthreads();
    // direction 0 (p -> i), lines (j, k): a1[p][j][k] -> out[e][i][j][k]
    for (int t = lt; t < NM2; t += NQ2) {
      V r[NQ];
#pragma unroll
      for (int p = 0; p < NQ; ++p) r[p] = a1[p * NM2 + t];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        Acc a;
        A::mul(a, sB[i], r[0]);
#pragma unroll
        for (int p = 1; p < NQ; ++p) A::fma(a, sB[p * NM + i], r[p]);
        if (!valid) continue;
        if (map) {  // scatter-add (atomic: DoFs shared between cells)
          const uint32_t d = __ldg(map + e * NM3 + i * NM2 + t);
          if (d != MFGB_INVALID_DOF) atomicAdd(out + d, A::store_vec(A::finish(a)));
        } else {
          out[e * NM3 + i * NM2 + t] = A::store_vec(A::finish(a));
        }
      }
    }
    __syncthreads();
  }
}

// BP3 operator (L-vector, NM = p + 1 GLL nodes interpolated to NQ Gauss points
// per direction; CEED_bp/include/bk3_kokkos_kernel.h:146-354) with the bulk-TMA
// pipeline of the BK5 kernels: G (6 x NQ^3 per cell, A::GType) and the dof map
// of the next batch stream into shared memory while this batch is computed,
// and the next gather is prefetched into registers.  A CTA holds E cells with
// NQ^2 threads per cell, thread (a, b) of a cell:
//   gather          (a, b) < NM: node column u[i][a][b]           -> W0
//   interp k        a < NM:  W1[i][a][q3 = b] = sum_m B[b][m] W0[i][a][m]
//   interp j, i     all:     t[i] = sum_m B[a][m] W1[i][m][b]; W0[q1][a][b] = sum_i B[q1][i] t[i]
//   gradient, metric         column (a, b), one Gauss point per step -> W3 (r), W1 (s), W2 (t)
//   integrate, back i        y[i] = sum_q1 B[q1][i] (D^T...)[q1]      -> W0 [i][a][b]
//   back j          a < NM:  W1[i][a][b] = sum_q2 B[q2][a] W0[i][q2][b]
//   back k, scatter (a, b) < NM: dst[map] += sum_q3 B[q3][b] W1[i][a][q3]
// The loops over the Gauss points of a column are not unrolled (values in
// shared memory, not registers): fully unrolled, the double-float code
// outgrew the instruction cache (warps stalled on instruction fetch).
// Every wait is bounded (a timeout sets err_flag and the CTA returns).
template <int NM, int NQ, class A>
struct BasisQ {
  typename A::V B[NQ * NM];  // B[q * NM + i] = l_i(g_q)
  typename A::V D[NQ * NQ];  // collocation derivative at the Gauss points
};

template <int NM, int NQ, int E, class A, int MB>
__global__ void __launch_bounds__(E * NQ * NQ, MB)
    bp3_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                   const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
                   typename A::VecT *__restrict__ dst, const BasisQ<NM, NQ, A> basis,
                   int *__restrict__ err_flag) {
  using V = typename A::V;
  using Acc = typename A::Acc;
  using GT = typename A::GType;
  using VT = typename A::VecT;
  using L = TmaLayoutQ<NM, NQ, E, A, 4>;
  constexpr int M2 = NM * NM, Q2 = NQ * NQ, Q3 = NQ * NQ * NQ, MQ = NM * NQ;
  extern __shared__ __align__(128) unsigned char smem[];
  GT *sG = reinterpret_cast<GT *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  V *w0 = reinterpret_cast<V *>(smem + L::g_bytes + L::map_bytes);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;
  __shared__ V sB[NQ * NM], sD[NQ * NQ];

  const int tid = threadIdx.x;
  const int el = tid / Q2;
  const int ab = tid - el * Q2;
  const int a = ab / NQ;
  const int b = ab - a * NQ;
  const bool node_col = a < NM && b < NM;  // owns a node column (gather / scatter)
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA
  V *W0 = w0 + el * Q3, *W1 = w0 + (E + el) * Q3, *W2 = w0 + (2 * E + el) * Q3,
    *W3 = w0 + (3 * E + el) * Q3;
  for (int q = tid; q < NQ * NM; q += blockDim.x) sB[q] = basis.B[q];
  for (int q = tid; q < NQ * NQ; q += blockDim.x) sD[q] = basis.D[q];

  const TmaTilesQ<NM, NQ, E, A> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
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
  uint32_t idx[NM];
  VT raw[NM];
  const int jk = node_col ? a * NM + b : 0;
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw, node_col);
  }

  for (; batch < n_batches; batch += gridDim.x) {
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase
    const bool valid = el < T.cells_of(batch);
    if (node_col) {
#pragma unroll
      for (int i = 0; i < NM; ++i)
        W0[i * M2 + jk] = idx[i] != MFGB_INVALID_DOF ? A::load_vec(raw[i]) : A::zero_v();
    }
    __syncthreads();  // barrier B: nodal values ready; the map tile is free
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }
    V c0[NQ], c1[NQ];
    // ---- interpolate along k: W1[i][a][b] (a < NM, b < NQ)
    if (a < NM) {
#pragma unroll
      for (int m = 0; m < NM; ++m) c0[m] = sB[b * NM + m];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        Acc s;
        A::mul(s, c0[0], W0[i * M2 + a * NM]);
#pragma unroll
        for (int m = 1; m < NM; ++m) A::fma(s, c0[m], W0[i * M2 + a * NM + m]);
        W1[i * MQ + a * NQ + b] = A::finish(s);
      }
    }
    __syncthreads();
    // ---- along j (shared) and i: the column's values at the Gauss points -> W0
    {
      V t[NM];
#pragma unroll
      for (int m = 0; m < NM; ++m) c0[m] = sB[a * NM + m];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        Acc s;
        A::mul(s, c0[0], W1[i * MQ + b]);
#pragma unroll
        for (int m = 1; m < NM; ++m) A::fma(s, c0[m], W1[i * MQ + m * NQ + b]);
        t[i] = A::finish(s);
      }
#pragma unroll 1
      for (int q = 0; q < NQ; ++q) {
        Acc s;
        A::mul(s, sB[q * NM], t[0]);
#pragma unroll
        for (int i = 1; i < NM; ++i) A::fma(s, sB[q * NM + i], t[i]);
        W0[q * Q2 + ab] = A::finish(s);
      }
    }
    __syncthreads();
    // ---- collocation gradient + metric (G tile in shared memory)
    const GT *Gc = sG + el * 6 * Q3 + ab;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      c0[m] = sD[a * NQ + m];
      c1[m] = sD[b * NQ + m];
    }
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      Acc ar, as, at;
      A::mul(ar, sD[q * NQ], W0[ab]);
      A::mul(as, c0[0], W0[q * Q2 + b]);
      A::mul(at, c1[0], W0[q * Q2 + a * NQ]);
#pragma unroll
      for (int m = 1; m < NQ; ++m) {
        A::fma(ar, sD[q * NQ + m], W0[m * Q2 + ab]);
        A::fma(as, c0[m], W0[q * Q2 + m * NQ + b]);
        A::fma(at, c1[m], W0[q * Q2 + a * NQ + m]);
      }
      const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
      V grr = A::zero_v(), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = A::load_g(Gc[0 * Q3 + q * Q2]);
        grs = A::load_g(Gc[1 * Q3 + q * Q2]);
        grt = A::load_g(Gc[2 * Q3 + q * Q2]);
        gss = A::load_g(Gc[3 * Q3 + q * Q2]);
        gst = A::load_g(Gc[4 * Q3 + q * Q2]);
        gtt = A::load_g(Gc[5 * Q3 + q * Q2]);
      }
      Acc br, bs, bt;
      A::mul(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::mul(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::mul(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      W3[q * Q2 + ab] = A::finish(br);
      W1[q * Q2 + ab] = A::finish(bs);
      W2[q * Q2 + ab] = A::finish(bt);
    }
    __syncthreads();  // barrier C: G tile consumed, W1 / W2 / W3 ready
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }
    // this batch's scatter targets; then prefetch the next batch's gather
    uint32_t cur[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) cur[i] = idx[i];
    if (has_next) {
      const bool okm = mbar_wait(mbar_m, ph_m);
      if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
      ph_m ^= 1u;
      if (okm) T.gather(next, el, jk, idx, raw, node_col);
      else
        for (int i = 0; i < NM; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = VT(0); }
    }
    // ---- integrate (D^T, sum of three) and back to the nodes along i
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      c0[m] = sD[m * NQ + a];
      c1[m] = sD[m * NQ + b];
    }
    Acc y[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) A::zero(y[i]);
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      Acc s;
      A::mul(s, sD[q], W3[ab]);
      A::fma(s, c0[0], W1[q * Q2 + b]);
      A::fma(s, c1[0], W2[q * Q2 + a * NQ]);
#pragma unroll
      for (int m = 1; m < NQ; ++m) {
        A::fma(s, sD[m * NQ + q], W3[m * Q2 + ab]);
        A::fma(s, c0[m], W1[q * Q2 + m * NQ + b]);
        A::fma(s, c1[m], W2[q * Q2 + a * NQ + m]);
      }
      const V tq = A::finish(s);
#pragma unroll
      for (int i = 0; i < NM; ++i) A::fma(y[i], sB[q * NM + i], tq);
    }
    // W0's last readers (the gradient) finished before barrier C
#pragma unroll
    for (int i = 0; i < NM; ++i) W0[i * Q2 + ab] = A::finish(y[i]);
    __syncthreads();  // W0 ready; W1, W2, W3 consumed
    // ---- back along j: W1[i][a][b] (a < NM)
    if (a < NM) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) c0[q] = sB[q * NM + a];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        Acc s;
        A::mul(s, c0[0], W0[i * Q2 + b]);
#pragma unroll
        for (int q = 1; q < NQ; ++q) A::fma(s, c0[q], W0[i * Q2 + q * NQ + b]);
        W1[i * MQ + a * NQ + b] = A::finish(s);
      }
    }
    __syncthreads();
    // ---- back along k and scatter-add (node columns)
    if (node_col) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) c0[q] = sB[q * NM + b];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        Acc s;
        A::mul(s, c0[0], W1[i * MQ + a * NQ]);
#pragma unroll
        for (int q = 1; q < NQ; ++q) A::fma(s, c0[q], W1[i * MQ + a * NQ + q]);
        if (cur[i] != MFGB_INVALID_DOF) atomicAdd(dst + cur[i], A::store_vec(A::finish(s)));
      }
    }
    // W1 is read above until barrier A of the next batch; W0 is rewritten only after it
  }
}

}  // namespace mfgb
