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
// GB300 structure: a CTA holds E elements, NQ^2 threads per element.  The
// interpolation passes run one 1D line per thread through shared memory; the
// Laplacian's gradient/metric/integrate phase uses the BK5 column layout (thread
// (q, r) keeps the direction-0 column of its points in registers).  Arithmetic
// is FP64 or double-float (policy A).
#pragma once
#include "mfgb_common.cuh"

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
        A::zero(a);
#pragma unroll
        for (int i = 0; i < NM; ++i) A::fma(a, sB[p * NM + i], r[i]);
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
        A::zero(a);
#pragma unroll
        for (int j = 0; j < NM; ++j) A::fma(a, sB[q * NM + j], r[j]);
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
        A::zero(a);
#pragma unroll
        for (int k = 0; k < NM; ++k) A::fma(a, sB[rr * NM + k], r[k]);
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
        A::zero(ar);
        A::zero(as);
        A::zero(at);
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
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
        A::zero(br);
        A::zero(bs);
        A::zero(bt);
        A::fma(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
        A::fma(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
        A::fma(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
        vr[p] = A::finish(br);
        a2[p * NQ2 + lt] = A::finish(bs);
        a3[p * NQ2 + lt] = A::finish(bt);
      }
      __syncthreads();  // a1 is no longer read: it receives the integrated values
#pragma unroll
      for (int p = 0; p < NQ; ++p) {
        Acc a;
        A::zero(a);
#pragma unroll
        for (int m = 0; m < NQ; ++m) {
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
        A::zero(a);
#pragma unroll
        for (int rr = 0; rr < NQ; ++rr) A::fma(a, sB[rr * NM + k], r[rr]);
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
        A::zero(a);
#pragma unroll
        for (int q = 0; q < NQ; ++q) A::fma(a, sB[q * NM + j], r[q]);
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
        A::zero(a);
#pragma unroll
        for (int p = 0; p < NQ; ++p) A::fma(a, sB[p * NM + i], r[p]);
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

}  // namespace mfgb
