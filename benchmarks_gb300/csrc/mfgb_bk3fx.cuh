// mfgb_bk3fx.cuh -- FP64-accurate CEED BK3 Laplacian on E-vectors (NM = p + 1
// modes to NQ = p + 2 points, out_e = B^T D^T G_e D B in_e; reference
// CEED_BK/include/kernels/BK3/serial_kernels.hpp:29-188) with the offset
// double-float accumulation of the BP3 kernel (mfgb_bp3fx.cuh).  The caller's
// FP64 G[e][6][nq^3] arrives by bulk copies; each element's largest G exponent
// is reduced in shared memory and the metric stage converts G to pairs scaled
// by it as it reads them, so any input range is carried.  Input and output are
// contiguous E-vectors (plain loads and stores, no dof map, no atomics).
#pragma once
#include "mfgb_bp3fx.cuh"

namespace mfgb {

template <int NM, int NQ, int E, int MB>
__global__ void __launch_bounds__(E * NQ * NQ, MB)
    bk3fx_tma_kernel(const int64_t n_cells, const double *__restrict__ G,
                     const double *__restrict__ src, double *__restrict__ dst,
                     const BasisQFX<NM, NQ> basis, int *__restrict__ err_flag) {
  using L = TmaLayoutQ<NM, NQ, E, ArithF64, 4>;
  constexpr int M2 = NM * NM, Q2 = NQ * NQ, Q3 = NQ * NQ * NQ, MQ = NM * NQ;
  extern __shared__ __align__(128) unsigned char smem[];
  double *sG = reinterpret_cast<double *>(smem);
  df *w0 = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar;
  __shared__ float2 sB[NQ * NM], sD[NQ * NQ];
  __shared__ float s_rB[NQ], s_cB[NM], s_rD[NQ], s_cD[NQ];
  __shared__ int s_emax[2][E];
  __shared__ unsigned s_w0max[E];
  __shared__ int s_gmax[E];  // largest biased exponent of the element's G

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
  if (tid < E) s_w0max[tid] = 0u, s_gmax[tid] = 0;
  const float LB = basis.LB;

  // the G tiles (FP64, the caller's array) by bulk copies; no dof map
  TmaTilesQ<NM, NQ, E, ArithF64> T{n_cells, nullptr, G, src, sG, nullptr, mbar_g, nullptr};
  auto fail = [&](uint32_t pg) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded wait for the copy still in flight
  };
  if (tid == 0) {
    mbar_init(mbar_g, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) T.issue_g(batch);
  uint32_t ph_g = 0;
  double raw[NM];
  const int jk = node_col ? a * NM + b : 0;
  // this thread's node column of element e of batch bt (E-vector: contiguous)
  auto load = [&](int64_t bt) {
    const int64_t e = bt * E + el;
    const bool ok = node_col && e < n_cells;
#pragma unroll
    for (int i = 0; i < NM; ++i) raw[i] = ok ? __ldg(src + e * M2 * NM + i * M2 + jk) : 0.0;
  };
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < NM; ++i) em = max(em, dexp(raw[i]));
    if (em) atomicMax(&s_emax[slot][el], em);
  };
  load(batch);
  reduce_exp(0);

  for (int it = 0; batch < n_batches; batch += gridDim.x, ++it) {
    const int slot = it & 1;
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // (every G tile arrives by bulk copy)
    const bool valid = el < T.cells_of(batch);
    const double *Gd = sG + el * 6 * Q3 + ab;
    if (valid) {  // the element's largest G exponent (read after barrier B)
      int eg = 0;
#pragma unroll 1
      for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int q = 0; q < NQ; ++q) eg = max(eg, dexp(Gd[c * Q3 + q * Q2]));
      if (eg) atomicMax(&s_gmax[el], eg);
    }
    const int su = fx_offset(s_emax[slot][el]);
    if (node_col) {
#pragma unroll
      for (int i = 0; i < NM; ++i) W0[i * M2 + jk] = fx_from_double(raw[i], su);
    }
    __syncthreads();  // barrier B: nodal values and s_gmax ready; s_emax[slot] read
    const int sg = fx_offset(s_gmax[el]);
    const int sc = su + sg;  // the element's result scale
    if (ab == 0) s_emax[slot][el] = 0;  // next written two batches on
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
    // G converted to scaled pairs as it is read (2^-sg for the element)
    auto gpair = [&](int c, int q) {
      const df d = fx_from_double(Gd[c * Q3 + q * Q2], sg);
      return make_float2(d.hi, d.lo);
    };
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
        grr = gpair(0, q);
        grs = gpair(1, q);
        grt = gpair(2, q);
        gss = gpair(3, q);
        gst = gpair(4, q);
        gtt = gpair(5, q);
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
    __syncthreads();  // barrier C: G tile consumed, W1 / W2 / W3 ready; s_w0max, s_gmax read
    if (ab == 0) s_w0max[el] = 0u, s_gmax[el] = 0;
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }
    const int64_t e_out = batch * E + el;  // this batch's element of the thread
    if (has_next) load(next);  // the next batch's nodes, used after its barrier A
    // ---- integrate (D^T, sum of three) and back to the nodes along i
#pragma unroll
    for (int m = 0; m < NQ; ++m) {
      const float2 u = sD[m * NQ + a], v = sD[m * NQ + b];
      c0h[m] = u.x, c0l[m] = u.y, c1h[m] = v.x, c1l[m] = v.y;
    }
    // bound of t_q: colsum|D| times the largest |value| of the own column (r)
    // and of the s- and t-lines it reads
    float tmax = 0.f;
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
      const float Cq = s_cD[q] * v3max + s_cD[a] * ms + s_cD[b] * mt;
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
        if (e_out < n_cells)
          dst[e_out * M2 * NM + i * M2 + jk] = fast_out ? fx_f2d_fast(yv.hi, kout) + fx_f2d_fast(yv.lo, kout)
                                                        : fx_f2d(yv.hi, sc) + fx_f2d(yv.lo, sc);
      }
    }
    // the next batch's largest exponent per element (read after its barrier A);
    // W1 is read above until that barrier
    if (has_next) reduce_exp(slot ^ 1);
  }
}

}  // namespace mfgb
