// mfgb_bp3fx.cuh -- FP64-accurate BP3 operator (L-vector, NM = p + 1 GLL nodes
// interpolated to NQ = p + 2 Gauss points per direction; reference
// CEED_bp/include/bk3_kokkos_kernel.h:146-354), and with NQ = p + 1 the Gauss
// form of the BP5 Laplacian (bakeoff_problems_dealii/include/
// portable_laplace_operator.h, QGauss(p+1)), on the FP32 pipes with the
// offset accumulation and per-cell exponent scaling of the collocation kernel
// (mfgb_bk5fx.cuh), in the bulk-TMA pipeline of bp3_tma_kernel (mfgb_bkq.cuh).
//
// Every dot product starts its offset accumulator at a bound C >= 2 sum |x y|:
//   interpolation along k and j (the gathered nodes scaled to |u| < 1 per
//     cell): K rowsum|B[q]| LB^s (LB = max_q rowsum|B[q]|, s = the
//     interpolations already applied); along i: K rowsum|B[q]| times the
//     column's largest input
//   gradient: K rowsum|D[q]| times the largest value of the own column (r) or
//     of the cell at the Gauss points (s, t; one shared atomicMax per thread)
//   metric: per point, K max|q| times the row sums of |G| (G pairs pre-scaled
//     per cell by 2^-sg)
//   integrate and the backward interpolations: K colsum|D| or K colsum|B|
//     times the largest |value| of each line read (the own column's, or the
//     line loaded into registers first); the Helmholtz form's mass term adds
//     K |JxW u| at the point (JxW pairs on the cell's G scale).
// The cell's result is scaled back by 2^(su + sg) when converted to double.
#pragma once
#include "mfgb_bk5fx.cuh"

namespace mfgb {

template <int NM, int NQ>
struct BasisQFX {
  float Bh[NQ * NM], Bl[NQ * NM];  // B[q * NM + i] = l_i(g_q) as a float pair
  float Dh[NQ * NQ], Dl[NQ * NQ];  // collocation derivative at the Gauss points
  float rB[NQ];                    // K sum_i |Bh[q][i]|
  float cB[NM];                    // K sum_q |Bh[q][i]|
  float rD[NQ];                    // K sum_m |Dh[q][m]|
  float cD[NQ];                    // K sum_q |Dh[q][m]|
  float LB;                        // max_q sum_i |Bh[q][i]|
  float K;
};

// largest |hi| of a float pair as ordered bits (non-negative floats order as
// unsigned integers), for shared atomicMax
__device__ __forceinline__ unsigned abs_bits(float x) { return __float_as_uint(fabsf(x)); }

// MASS: the Helmholtz form's mass term JxW u at every Gauss point (jxw: the
// JxW pairs [cell][NQ^3] on the cell's G scale), each point's value loaded one
// point ahead of its use
template <int NM, int NQ, int E, int MB, bool MAPTMA, bool MASS = false>
__global__ void __launch_bounds__(E * NQ * NQ, MB)
    bp3fx_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                     const float2 *__restrict__ G, const int *__restrict__ gexp,
                     const double *__restrict__ src, double *__restrict__ dst,
                     const BasisQFX<NM, NQ> basis, const int *__restrict__ done_flag,
                     int *__restrict__ err_flag, const float2 *__restrict__ jxw) {
  if (done_flag != nullptr && *done_flag) return;
  using L = TmaLayoutQ<NM, NQ, E, ArithDF, 4>;
  constexpr int M2 = NM * NM, Q2 = NQ * NQ, Q3 = NQ * NQ * NQ, MQ = NM * NQ;
  extern __shared__ __align__(128) unsigned char smem[];
  float2 *sG = reinterpret_cast<float2 *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  df *w0 = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;
  __shared__ float2 sB[NQ * NM], sD[NQ * NQ];
  __shared__ float s_rB[NQ], s_cB[NM], s_rD[NQ], s_cD[NQ];
  __shared__ int s_emax[2][E];
  __shared__ unsigned s_w0max[E];

  const int tid = threadIdx.x;
  const int el = tid / Q2;
  const int ab = tid - el * Q2;
  const int a = ab / NQ;
  const int b = ab - a * NQ;
  const bool node_col = a < NM && b < NM;  // owns a node column (gather / scatter)
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA
  df *W0 = w0 + el * Q3, *W1 = w0 + (E + el) * Q3, *W2 = w0 + (2 * E + el) * Q3,
     *W3 = w0 + (3 * E + el) * Q3;
  for (int q = tid; q < NQ * NM; q += blockDim.x) sB[q] = make_float2(basis.Bh[q], basis.Bl[q]);
  for (int q = tid; q < NQ * NQ; q += blockDim.x) sD[q] = make_float2(basis.Dh[q], basis.Dl[q]);
  for (int q = tid; q < NQ; q += blockDim.x) {
    s_rB[q] = basis.rB[q];
    s_rD[q] = basis.rD[q];
    s_cD[q] = basis.cD[q];
  }
  for (int q = tid; q < NM; q += blockDim.x) s_cB[q] = basis.cB[q];
  if (tid < 2 * E) (&s_emax[0][0])[tid] = 0;
  if (tid < E) s_w0max[tid] = 0u;
  const float LB = basis.LB;

  TmaTilesQ<NM, NQ, E, ArithDF> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  T.map_ok = MAPTMA;
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
  double raw[NM];
  int ge = 0;  // G exponent offset of this thread's cell in the prefetched batch
  const int jk = node_col ? a * NM + b : 0;
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < NM; ++i) em = max(em, idx[i] != MFGB_INVALID_DOF ? dexp(raw[i]) : 0);
    if (em) atomicMax(&s_emax[slot][el], em);
  };
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw, node_col);
    reduce_exp(0);
    if (el < T.cells_of(batch)) ge = __ldg(gexp + batch * E + el);
  }

  for (int it = 0; batch < n_batches; batch += gridDim.x, ++it) {
    const int slot = it & 1;
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase
    const bool valid = el < T.cells_of(batch);
    const int su = fx_offset(s_emax[slot][el]);
    const int sc = su + ge;  // the cell's result scale
    if (node_col) {
#pragma unroll
      for (int i = 0; i < NM; ++i)
        W0[i * M2 + jk] = idx[i] != MFGB_INVALID_DOF ? fx_from_double(raw[i], su) : df{0.f, 0.f};
    }
    __syncthreads();  // barrier B: nodal values ready; s_emax[slot] read; the map tile is free
    if (ab == 0) s_emax[slot][el] = 0;  // next written two batches on
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }
    float c0h[NQ], c0l[NQ], c1h[NQ], c1l[NQ];
    float w0col = 0.f;
    // ---- interpolate along k: W1[i][a][b] (a < NM, b < NQ), |W0| < 1
    if (a < NM) {
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        const float2 c = sB[b * NM + m];
        c0h[m] = c.x, c0l[m] = c.y;
      }
      const float C = s_rB[b];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        fxacc s;
        const df v0 = W0[i * M2 + a * NM];
        fx_first(s, c0h[0], c0l[0], v0.hi, v0.lo, C);
#pragma unroll
        for (int m = 1; m < NM; ++m) {
          const df v = W0[i * M2 + a * NM + m];
          fx_fma(s, c0h[m], c0l[m], v.hi, v.lo);
        }
        W1[i * MQ + a * NQ + b] = fx_finish(s, C);
      }
    }
    __syncthreads();
    // ---- along j (shared) and i: the column's values at the Gauss points -> W0
    {
      df t[NM];
#pragma unroll
      for (int m = 0; m < NM; ++m) {
        const float2 c = sB[a * NM + m];
        c0h[m] = c.x, c0l[m] = c.y;
      }
      const float Cj = s_rB[a] * LB;
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        fxacc s;
        const df v0 = W1[i * MQ + b];
        fx_first(s, c0h[0], c0l[0], v0.hi, v0.lo, Cj);
#pragma unroll
        for (int m = 1; m < NM; ++m) {
          const df v = W1[i * MQ + m * NQ + b];
          fx_fma(s, c0h[m], c0l[m], v.hi, v.lo);
        }
        t[i] = fx_finish(s, Cj);
      }
      float tm = 0.f;
#pragma unroll
      for (int i = 0; i < NM; ++i) tm = fmaxf(tm, fabsf(t[i].hi));
      float gmax = 0.f;  // this column's largest value at the Gauss points
#pragma unroll 1
      for (int q = 0; q < NQ; ++q) {
        const float Ci = s_rB[q] * tm;
        fxacc s;
        const float2 c = sB[q * NM];
        fx_first(s, c.x, c.y, t[0].hi, t[0].lo, Ci);
#pragma unroll
        for (int i = 1; i < NM; ++i) {
          const float2 ci = sB[q * NM + i];
          fx_fma(s, ci.x, ci.y, t[i].hi, t[i].lo);
        }
        const df w = fx_finish(s, Ci);
        W0[q * Q2 + ab] = w;
        gmax = fmaxf(gmax, fabsf(w.hi));
      }
      if (gmax > 0.f) atomicMax(&s_w0max[el], abs_bits(gmax));
      w0col = gmax;
    }
    __syncthreads();  // W0 at the Gauss points and s_w0max ready
    // ---- collocation gradient + metric (scaled G pairs in shared memory)
    const float2 *Gc = sG + el * 6 * Q3 + ab;
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      const float2 u = sD[a * NQ + m], v = sD[b * NQ + m];
      c0h[m] = u.x, c0l[m] = u.y, c1h[m] = v.x, c1l[m] = v.y;
    }
    // gradient bounds: the own column (r) and the cell (s, t) at the Gauss points
    const float w0cell = __uint_as_float(s_w0max[el]);
    const float Cs = s_rD[a] * w0cell, Ct = s_rD[b] * w0cell;
    float v3max = 0.f;  // this column's largest |W3|
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      const float Cr = s_rD[q] * w0col;
      fxacc ar, as, at;
      {
        const float2 d = sD[q * NQ];
        const df x = W0[ab], y = W0[q * Q2 + b], z = W0[q * Q2 + a * NQ];
        fx_first(ar, d.x, d.y, x.hi, x.lo, Cr);
        fx_first(as, c0h[0], c0l[0], y.hi, y.lo, Cs);
        fx_first(at, c1h[0], c1l[0], z.hi, z.lo, Ct);
      }
#pragma unroll
      for (int m = 1; m < NQ; ++m) {
        const float2 d = sD[q * NQ + m];
        const df x = W0[m * Q2 + ab], y = W0[q * Q2 + m * NQ + b], z = W0[q * Q2 + a * NQ + m];
        fx_fma(ar, d.x, d.y, x.hi, x.lo);
        fx_fma(as, c0h[m], c0l[m], y.hi, y.lo);
        fx_fma(at, c1h[m], c1l[m], z.hi, z.lo);
      }
      const df qr = fx_finish(ar, Cr), qs = fx_finish(as, Cs), qt = fx_finish(at, Ct);
      float2 grr = make_float2(0.f, 0.f), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = Gc[0 * Q3 + q * Q2];
        grs = Gc[1 * Q3 + q * Q2];
        grt = Gc[2 * Q3 + q * Q2];
        gss = Gc[3 * Q3 + q * Q2];
        gst = Gc[4 * Q3 + q * Q2];
        gtt = Gc[5 * Q3 + q * Q2];
      }
      const float kq = basis.K * fmaxf(fmaxf(fabsf(qr.hi), fabsf(qs.hi)), fabsf(qt.hi));
      const float Br = (fabsf(grr.x) + fabsf(grs.x) + fabsf(grt.x)) * kq;
      const float Bs = (fabsf(grs.x) + fabsf(gss.x) + fabsf(gst.x)) * kq;
      const float Bt = (fabsf(grt.x) + fabsf(gst.x) + fabsf(gtt.x)) * kq;
      fxacc br, bs, bt;
      fx_first(br, grr.x, grr.y, qr.hi, qr.lo, Br);
      fx_fma(br, grs.x, grs.y, qs.hi, qs.lo);
      fx_fma(br, grt.x, grt.y, qt.hi, qt.lo);
      fx_first(bs, grs.x, grs.y, qr.hi, qr.lo, Bs);
      fx_fma(bs, gss.x, gss.y, qs.hi, qs.lo);
      fx_fma(bs, gst.x, gst.y, qt.hi, qt.lo);
      fx_first(bt, grt.x, grt.y, qr.hi, qr.lo, Bt);
      fx_fma(bt, gst.x, gst.y, qs.hi, qs.lo);
      fx_fma(bt, gtt.x, gtt.y, qt.hi, qt.lo);
      const df vr = fx_finish(br, Br), vs = fx_finish(bs, Bs), vt = fx_finish(bt, Bt);
      W3[q * Q2 + ab] = vr;
      W1[q * Q2 + ab] = vs;
      W2[q * Q2 + ab] = vt;
      v3max = fmaxf(v3max, fabsf(vr.hi));
    }
    __syncthreads();  // barrier C: G tile consumed, W1 / W2 / W3 ready; s_w0max read
    if (ab == 0) s_w0max[el] = 0u;
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
      if (okm) {
        T.gather(next, el, jk, idx, raw, node_col);
      } else {
#pragma unroll
        for (int i = 0; i < NM; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = 0.0; }
      }
      ge = el < T.cells_of(next) ? __ldg(gexp + next * E + el) : 0;
    }
    // ---- integrate (D^T, sum of three) and back to the nodes along i
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      const float2 u = sD[m * NQ + a], v = sD[m * NQ + b];
      c0h[m] = u.x, c0l[m] = u.y, c1h[m] = v.x, c1l[m] = v.y;
    }
    // bound of t_q: colsum|D| times the largest |value| of the own column (r)
    // and of the s- and t-lines it reads
    float tmax = 0.f;
    const float2 *jxc = MASS ? jxw + (batch * E + el) * Q3 + ab : nullptr;  // this column's JxW
    float2 jw_next = make_float2(0.f, 0.f);
    if (MASS && valid) jw_next = __ldg(jxc);
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      df ls[NQ], lt[NQ];
      float ms = 0.f, mt = 0.f;
#pragma unroll
      for (int m = 0; m < NQ; ++m) {
        ls[m] = W1[q * Q2 + m * NQ + b];
        lt[m] = W2[q * Q2 + a * NQ + m];
        ms = fmaxf(ms, fabsf(ls[m].hi));
        mt = fmaxf(mt, fabsf(lt[m].hi));
      }
      // the mass term JxW u at the point (u: the own column's value at the
      // Gauss point, still in W0)
      float2 jw = make_float2(0.f, 0.f);
      df uq = {0.f, 0.f};
      if (MASS) {
        jw = jw_next;
        if (valid && q + 1 < NQ) jw_next = __ldg(jxc + (q + 1) * Q2);
        uq = W0[q * Q2 + ab];
      }
      const float Cq = s_cD[q] * v3max + s_cD[a] * ms + s_cD[b] * mt +
                       basis.K * fabsf(jw.x) * fabsf(uq.hi);
      fxacc s;
      {
        const float2 d = sD[q];
        const df x = W3[ab];
        fx_first(s, d.x, d.y, x.hi, x.lo, Cq);
        fx_fma(s, c0h[0], c0l[0], ls[0].hi, ls[0].lo);
        fx_fma(s, c1h[0], c1l[0], lt[0].hi, lt[0].lo);
      }
#pragma unroll
      for (int m = 1; m < NQ; ++m) {
        const float2 d = sD[m * NQ + q];
        const df x = W3[m * Q2 + ab];
        fx_fma(s, d.x, d.y, x.hi, x.lo);
        fx_fma(s, c0h[m], c0l[m], ls[m].hi, ls[m].lo);
        fx_fma(s, c1h[m], c1l[m], lt[m].hi, lt[m].lo);
      }
      if (MASS) fx_fma(s, jw.x, jw.y, uq.hi, uq.lo);
      const df tq = fx_finish(s, Cq);
      W0[q * Q2 + ab] = tq;  // the own column; W0's last readers (the gradient) were before barrier C
      tmax = fmaxf(tmax, fabsf(tq.hi));
    }
    // back along i with the column's own bound
    fxacc y[NM];
    float Cy[NM];
#pragma unroll
    for (int i = 0; i < NM; ++i) {
      Cy[i] = basis.cB[i] * tmax;
      y[i].T = Cy[i];
      y[i].S = 0.f;
    }
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      const df tq = W0[q * Q2 + ab];
#pragma unroll
      for (int i = 0; i < NM; ++i) {
        const float2 c = sB[q * NM + i];
        fx_fma(y[i], c.x, c.y, tq.hi, tq.lo);
      }
    }
#pragma unroll
    for (int i = 0; i < NM; ++i) W0[i * Q2 + ab] = fx_finish(y[i], Cy[i]);
    __syncthreads();  // barrier D: W0 ready; W1, W2, W3 consumed
    // ---- back along j: W1[i][a][b] (a < NM), bound from the line read
    if (a < NM) {
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float2 c = sB[q * NM + a];
        c0h[q] = c.x, c0l[q] = c.y;
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
        fx_first(s, c0h[0], c0l[0], l[0].hi, l[0].lo, C);
#pragma unroll
        for (int q = 1; q < NQ; ++q) fx_fma(s, c0h[q], c0l[q], l[q].hi, l[q].lo);
        W1[i * MQ + a * NQ + b] = fx_finish(s, C);
      }
    }
    __syncthreads();  // barrier E: W1 ready
    // ---- back along k and scatter-add (node columns)
    if (node_col) {
      const bool fast_out = (unsigned)(sc + 896) <= 1792u;
      const unsigned kout = (unsigned)(896 + sc) << 20;
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float2 c = sB[q * NM + b];
        c0h[q] = c.x, c0l[q] = c.y;
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
        fx_first(s, c0h[0], c0l[0], l[0].hi, l[0].lo, C);
#pragma unroll
        for (int q = 1; q < NQ; ++q) fx_fma(s, c0h[q], c0l[q], l[q].hi, l[q].lo);
        const df yv = fx_finish(s, C);
        if (cur[i] != MFGB_INVALID_DOF)
          atomicAdd(dst + cur[i], fast_out ? fx_f2d_fast(yv.hi, kout) + fx_f2d_fast(yv.lo, kout)
                                           : fx_f2d(yv.hi, sc) + fx_f2d(yv.lo, sc));
      }
    }
    // the prefetched gather's largest exponent per cell (read after the next
    // barrier A); W1 is read above until barrier A of the next batch
    if (has_next) reduce_exp(slot ^ 1);
  }
}

}  // namespace mfgb
