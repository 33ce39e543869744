// mfgb_bk1fx.cuh -- FP64-accurate CEED BK1 mass operator on E-vectors
// (out_e = B^T (JxW_e o (B x B x B) in_e), NM = p + 1 modes to NQ = p + 2
// points; reference CEED_BK/include/kernels/BK1/serial_kernels.hpp:20-121) on
// the FP32 pipes with the offset accumulation of the collocation kernel
// (mfgb_bk5fx.cuh) and per-element exponent scaling of the input and of JxW.
//
// A CTA holds E elements, NQ^2 threads per element, thread (a, b):
//   interpolation along k (a < NM):  W1[i][a][q3 = b] = sum_m B[b][m] W0[i][a][m]
//   along j and i, in registers:     t[i] = sum_m B[a][m] W1[i][m][b];
//                                    g[q] = sum_i B[q][i] t[i]
//   JxW and back along i:            y[i] = sum_q B[q][i] (JxW[q][a][b] g[q]) -> W0
//   back along j (a < NM):           W1[i][a][b] = sum_q B[q][a] W0[i][q][b]
//   back along k, store (node col):  out[i][a][b] = sum_q B[q][b] W1[i][a][q]
// The element's input (node columns) and JxW (all columns) of the next batch
// are loaded into registers during the current one.  Bounds of the offset
// accumulators: forward K rowsum|B| LB^s (|u| < 1 after scaling), the
// column's own largest value where the column is in registers, and the
// largest |value| of each line read from shared memory.
#pragma once
#include "mfgb_bp3fx.cuh"

namespace mfgb {

template <int NM, int NQ, int E, int MB>
__global__ void __launch_bounds__(E * NQ * NQ, MB)
    bk1fx_kernel(const int64_t nelmt, const double *__restrict__ in,
                 const double *__restrict__ JxW, double *__restrict__ out,
                 const BasisQFX<NM, NQ> basis) {
  constexpr int M2 = NM * NM, M3 = M2 * NM, Q2 = NQ * NQ, Q3 = Q2 * NQ, MQ = NM * NQ;
  __shared__ df W0s[E * NM * Q2], W1s[E * NM * MQ];
  __shared__ float2 sB[NQ * NM];
  __shared__ float s_rB[NQ], s_cB[NM];
  __shared__ int s_emax[2][E], s_jmax[2][E];

  const int tid = threadIdx.x;
  const int el = tid / Q2;
  const int ab = tid - el * Q2;
  const int a = ab / NQ;
  const int b = ab - a * NQ;
  const bool node_col = a < NM && b < NM;
  const int jk = node_col ? a * NM + b : 0;
  const int64_t n_batches = (nelmt + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA
  df *W0 = W0s + el * NM * Q2, *W1 = W1s + el * NM * MQ;
  for (int q = tid; q < NQ * NM; q += blockDim.x) sB[q] = make_float2(basis.Bh[q], basis.Bl[q]);
  for (int q = tid; q < NQ; q += blockDim.x) s_rB[q] = basis.rB[q];
  for (int q = tid; q < NM; q += blockDim.x) s_cB[q] = basis.cB[q];
  if (tid < 2 * E) {
    (&s_emax[0][0])[tid] = 0;
    (&s_jmax[0][0])[tid] = 0;
  }
  const float LB = basis.LB;
  __syncthreads();

  double raw[NM], jraw[NQ];
  auto load = [&](int64_t bt) {
    const int64_t e = bt * E + el;
    const bool valid = e < nelmt;
#pragma unroll
    for (int i = 0; i < NM; ++i) raw[i] = valid && node_col ? __ldg(in + e * M3 + i * M2 + jk) : 0.0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) jraw[q] = valid ? __ldg(JxW + e * Q3 + q * Q2 + ab) : 0.0;
  };
  auto reduce_exp = [&](int slot) {
    int eu = 0, ej = 0;
#pragma unroll
    for (int i = 0; i < NM; ++i) eu = max(eu, dexp(raw[i]));
#pragma unroll
    for (int q = 0; q < NQ; ++q) ej = max(ej, dexp(jraw[q]));
    if (eu) atomicMax(&s_emax[slot][el], eu);
    if (ej) atomicMax(&s_jmax[slot][el], ej);
  };
  load(batch);
  reduce_exp(0);

  for (int it = 0; batch < n_batches; batch += gridDim.x, ++it) {
    const int slot = it & 1;
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const int64_t e = batch * E + el;
    __syncthreads();  // the exponents of this batch are in; W0 / W1 free
    const int su = fx_offset(s_emax[slot][el]), sj = fx_offset(s_jmax[slot][el]);
    const int sc = su + sj;  // the element's result scale
    df jx[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) jx[q] = fx_from_double(jraw[q], sj);
    if (node_col) {
#pragma unroll
      for (int i = 0; i < NM; ++i) W0[i * M2 + jk] = fx_from_double(raw[i], su);
    }
    __syncthreads();  // nodal values ready; s_emax / s_jmax [slot] read
    if (ab == 0) s_emax[slot][el] = s_jmax[slot][el] = 0;  // next written two batches on
    if (has_next) load(next);
    float ch[NQ], cl[NQ];
    // ---- interpolate along k: W1[i][a][b] (a < NM, b < NQ), |W0| < 1
    if (a < NM) {
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        const float2 c = sB[b * NM + m];
        ch[m] = c.x, cl[m] = c.y;
      }
      const float C = s_rB[b];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        fxacc s;
        const df v0 = W0[i * M2 + a * NM];
        fx_first(s, ch[0], cl[0], v0.hi, v0.lo, C);
#pragma unroll
        for (int m = 1; m < NM; ++m) {
          const df v = W0[i * M2 + a * NM + m];
          fx_fma(s, ch[m], cl[m], v.hi, v.lo);
        }
        W1[i * MQ + a * NQ + b] = fx_finish(s, C);
      }
    }
    __syncthreads();
    // ---- along j (shared) and i (registers), JxW, back along i (registers)
    {
      df t[NM];
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        const float2 c = sB[a * NM + m];
        ch[m] = c.x, cl[m] = c.y;
      }
      const float Cj = s_rB[a] * LB;
      float tm = 0.f;
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        fxacc s;
        const df v0 = W1[i * MQ + b];
        fx_first(s, ch[0], cl[0], v0.hi, v0.lo, Cj);
#pragma unroll
        for (int m = 1; m < NM; ++m) {
          const df v = W1[i * MQ + m * NQ + b];
          fx_fma(s, ch[m], cl[m], v.hi, v.lo);
        }
        t[i] = fx_finish(s, Cj);
        tm = fmaxf(tm, fabsf(t[i].hi));
      }
      df w[NQ];  // JxW times the values at the points of the column
      float wm = 0.f;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float Ci = basis.rB[q] * tm;
        fxacc s;
        fx_first(s, basis.Bh[q * NM], basis.Bl[q * NM], t[0].hi, t[0].lo, Ci);
#pragma unroll
        for (int i = 1; i < NM; ++i) fx_fma(s, basis.Bh[q * NM + i], basis.Bl[q * NM + i], t[i].hi, t[i].lo);
        const df g = fx_finish(s, Ci);
        const float Cw = basis.K * fabsf(jx[q].hi) * fabsf(g.hi);
        fxacc m;
        fx_first(m, jx[q].hi, jx[q].lo, g.hi, g.lo, Cw);
        w[q] = fx_finish(m, Cw);
        wm = fmaxf(wm, fabsf(w[q].hi));
      }
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        const float Cy = basis.cB[i] * wm;
        fxacc s;
        fx_first(s, basis.Bh[i], basis.Bl[i], w[0].hi, w[0].lo, Cy);
#pragma unroll
        for (int q = 1; q < NQ; ++q) fx_fma(s, basis.Bh[q * NM + i], basis.Bl[q * NM + i], w[q].hi, w[q].lo);
        W0[i * Q2 + ab] = fx_finish(s, Cy);
      }
    }
    __syncthreads();  // W0[i][q1][q2] ready; W1 consumed
    // ---- back along j: W1[i][a][b] (a < NM), bound from the line read
    if (a < NM) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float2 c = sB[q * NM + a];
        ch[q] = c.x, cl[q] = c.y;
      }
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        df l[NQ];
        float ml = 0.f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          l[q] = W0[i * Q2 + q * NQ + b];
          ml = fmaxf(ml, fabsf(l[q].hi));
        }
        const float C = s_cB[a] * ml;
        fxacc s;
        fx_first(s, ch[0], cl[0], l[0].hi, l[0].lo, C);
#pragma unroll
        for (int q = 1; q < NQ; ++q) fx_fma(s, ch[q], cl[q], l[q].hi, l[q].lo);
        W1[i * MQ + a * NQ + b] = fx_finish(s, C);
      }
    }
    __syncthreads();  // W1[i][a][q3] ready
    // ---- back along k and store (node columns)
    if (node_col && e < nelmt) {
      const bool fast_out = (unsigned)(sc + 896) <= 1792u;
      const unsigned kout = (unsigned)(896 + sc) << 20;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float2 c = sB[q * NM + b];
        ch[q] = c.x, cl[q] = c.y;
      }
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        df l[NQ];
        float ml = 0.f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          l[q] = W1[i * MQ + a * NQ + q];
          ml = fmaxf(ml, fabsf(l[q].hi));
        }
        const float C = s_cB[b] * ml;
        fxacc s;
        fx_first(s, ch[0], cl[0], l[0].hi, l[0].lo, C);
#pragma unroll
        for (int q = 1; q < NQ; ++q) fx_fma(s, ch[q], cl[q], l[q].hi, l[q].lo);
        const df y = fx_finish(s, C);
        out[e * M3 + i * M2 + jk] = fast_out ? fx_f2d_fast(y.hi, kout) + fx_f2d_fast(y.lo, kout)
                                             : fx_f2d(y.hi, sc) + fx_f2d(y.lo, sc);
      }
    }
    // the next batch's largest exponents per element (read after the next
    // barrier); W1 is read above until that barrier
    if (has_next) reduce_exp(slot ^ 1);
  }
}

}  // namespace mfgb
