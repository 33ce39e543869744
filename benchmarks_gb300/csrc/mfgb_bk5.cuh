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

template <int N, int E, class A, bool EVEC, bool WITH_ENERGY>
__global__ void __launch_bounds__(E * N * N)
    bk5_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
               const typename A::GType *__restrict__ G, const typename A::VecT *__restrict__ src,
               typename A::VecT *__restrict__ dst, const Basis<N, A> basis,
               double *__restrict__ energy_partials, const int *__restrict__ done_flag) {
  if (done_flag != nullptr && *done_flag) return;  // solver already finished
  using V = typename A::V;
  using Acc = typename A::Acc;
  constexpr int N2 = N * N, N3 = N * N * N;
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

    // ---- reference gradient + metric apply
    V vr[N];
    const typename A::GType *Gc = G + (valid ? cell : 0) * 6 * N3 + jk;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc ar, as, at;
      A::zero(ar);
      A::zero(as);
      A::zero(at);
#pragma unroll
      for (int m = 0; m < N; ++m) {
        A::fma(ar, basis.D[i * N + m], u[m]);
        A::fma(as, Dj[m], s_u[el * N3 + i * N2 + m * N + k]);
        A::fma(at, Dk[m], s_u[el * N3 + i * N2 + j * N + m]);
      }
      const V qr = A::finish(ar), qs = A::finish(as), qt = A::finish(at);
      const V grr = A::load_g(__ldg(Gc + 0 * N3 + i * N2));
      const V grs = A::load_g(__ldg(Gc + 1 * N3 + i * N2));
      const V grt = A::load_g(__ldg(Gc + 2 * N3 + i * N2));
      const V gss = A::load_g(__ldg(Gc + 3 * N3 + i * N2));
      const V gst = A::load_g(__ldg(Gc + 4 * N3 + i * N2));
      const V gtt = A::load_g(__ldg(Gc + 5 * N3 + i * N2));
      Acc br, bs, bt;
      A::zero(br);
      A::zero(bs);
      A::zero(bt);
      A::fma(br, grr, qr); A::fma(br, grs, qs); A::fma(br, grt, qt);
      A::fma(bs, grs, qr); A::fma(bs, gss, qs); A::fma(bs, gst, qt);
      A::fma(bt, grt, qr); A::fma(bt, gst, qs); A::fma(bt, gtt, qt);
      vr[i] = A::finish(br);
      s_vs[el * N3 + i * N2 + jk] = A::finish(bs);
      s_vt[el * N3 + i * N2 + jk] = A::finish(bt);
    }
    __syncthreads();

    // ---- integrate (D^T, sum of the three directions) + scatter
#pragma unroll
    for (int i = 0; i < N; ++i) {
      Acc a;
      A::zero(a);
#pragma unroll
      for (int m = 0; m < N; ++m) {
        A::fma(a, basis.D[m * N + i], vr[m]);
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

}  // namespace mfgb
