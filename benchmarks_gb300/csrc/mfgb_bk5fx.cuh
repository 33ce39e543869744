// mfgb_bk5fx.cuh -- FP64-accurate BK5 collocation operator on the FP32 pipes with
// offset ("fixed-exponent") double-float accumulation and per-cell exponent scaling.
//
// The operator is the one of bk5_tma_kernel (GLL collocation: gather through the
// dof map with the 0xFFFFFFFF mask, collocation gradient, symmetric metric G,
// transpose, atomic scatter; reference CEED_BK/include/kernels/BK5/
// templated_cuda_kernels.cuh:50-122 and bakeoff_problems_dealii/include/
// bk3_kokkos_kernel.h:129-151, 406-426) with the same bulk-TMA pipeline.  What
// differs is the arithmetic:
//
// * Scaling.  Every cell's gathered values are multiplied by 2^-su, su chosen
//   from the largest binary exponent among them so that |u| < 1, and the
//   geometric factors are stored pre-multiplied by a per-cell 2^-sg (|G| < 1;
//   sg in a per-cell int array).  The scalings are exact.  The cell's result is
//   multiplied by 2^(su + sg) when it is converted back to double, so any FP64
//   input range is carried (no float over- or underflow of the pairs).
//
// * Offset accumulation.  A dot product sum_k x_k y_k of double-float pairs is
//   accumulated as T + S with T started at an offset C >= 2 B, where B bounds
//   sum_k |x_k.hi y_k.hi|.  Every partial sum then keeps C/2 <= T <= 3C/2, so
//     T' = fma(x.hi, y.hi, T)     rounds the product into T,
//     d  = T' - T                 is exact (|T| >= |product|: Dekker's Fast2Sum),
//     r  = fma(x.hi, y.hi, -d)    is the rounding error of T' (to float precision),
//     S += (r + x.hi y.lo) + x.lo y.hi
//   and at the end hi = T - C is exact (Sterbenz), lo = S.  That is 6 FP32-pipe
//   instructions per multiply-add (5 for the first), against 12 for the
//   TwoSum-based form of ArithDF, with an error of about 2^-46 of C.  The bounds
//   B come from the data at hand: |u| < 1 for the gradient (B = sum_m |D[i][m]|),
//   max |q| times the row sum of |G| per point for the metric, and the line
//   maxima of |v| times the column sums of |D| for the transpose.
//
// A float32 restatement of this arithmetic with its error bound is in
// tests/test_fx_arith.py.
#pragma once
#include "mfgb_bk5.cuh"

namespace mfgb {

// D split into float pairs plus the bound factors of the two contractions:
//   cg[i] = K * sum_m |Dh[i][m]|  (gradient output i, |data| < 1)
//   ci[i] = K * sum_m |Dh[m][i]|  (transpose output i, per unit of line maximum)
//   K = 2 (1 + 2^-20): the factor 2 of the offset, plus a margin for the float
//   rounding of the bound itself
template <int N>
struct BasisFX {
  float Dh[N * N], Dl[N * N];
  float cg[N], ci[N];
  float K;
};

// offset accumulator: value = (T - C) + S
struct fxacc {
  float T, S;
};

__device__ __forceinline__ void fx_first(fxacc &a, float xh, float xl, float yh, float yl,
                                         float C) {
  a.T = __fmaf_rn(xh, yh, C);
  const float d = __fsub_rn(a.T, C);
  const float r = __fmaf_rn(xh, yh, -d);
  a.S = __fmaf_rn(xl, yh, __fmaf_rn(xh, yl, r));
}

// the low-order terms of one product (its rounding error and the two cross
// products) are summed first and join S with one addition: the two chains a
// sum carries (T and S) advance by one dependent instruction per term
__device__ __forceinline__ void fx_fma(fxacc &a, float xh, float xl, float yh, float yl) {
  const float t = __fmaf_rn(xh, yh, a.T);
  const float d = __fsub_rn(t, a.T);
  const float r = __fmaf_rn(xh, yh, -d);
  const float e = __fmaf_rn(xl, yh, __fmaf_rn(xh, yl, r));
  a.S = __fadd_rn(a.S, e);
  a.T = t;
}

__device__ __forceinline__ df fx_finish(const fxacc &a, float C) {
  df r;
  r.hi = __fsub_rn(a.T, C);
  r.lo = a.S;
  return r;
}

// biased binary exponent of a double (0 for zero and subnormals, 2047 for inf/NaN)
__device__ __forceinline__ int dexp(double x) {
  return (int)(((unsigned)(__double_as_longlong(x) >> 32) >> 20) & 0x7FFu);
}

// x * 2^-off as a float pair by integer operations (off chosen so that the
// cell's largest value lands in [0.5, 1)): hi = the top 24 significant bits,
// lo = the next 29 bits rounded to float.  Values below 2^-126 after scaling
// (126 binades under the cell's largest), zeros and double subnormals flush to
// zero; inf and NaN give NaN.
__device__ __forceinline__ df fx_from_double(double x, int off) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7FFu);
  df r;
  if (e == 0x7FF) { r.hi = __uint_as_float(0x7FC00000u); r.lo = 0.f; return r; }
  const int es = e - off;
  if (e == 0 || es <= 896) { r.hi = 0.f; r.lo = 0.f; return r; }
  const unsigned hm = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
  r.hi = __uint_as_float(sign | ((unsigned)(es - 896) << 23) | hm);
  const unsigned rem = lw & 0x1FFFFFFFu;
  if (rem == 0u || es < 949) {
    r.lo = 0.f;
  } else {
    const unsigned fb = __float_as_uint(__uint2float_rn(rem));
    r.lo = __uint_as_float(sign | (fb + ((unsigned)(es - 1075) << 23)));
  }
  return r;
}

// f * 2^sc as a double by integer operations; float subnormals -> 0, results
// outside the double range -> 0 or +-inf, inf/NaN kept
__device__ __forceinline__ double fx_f2d(float f, int sc) {
  const unsigned u = __float_as_uint(f);
  const int ex = (int)((u >> 23) & 0xFFu);
  const unsigned long long sgn = (unsigned long long)(u & 0x80000000u) << 32;
  if (ex == 0) return 0.0;
  if (ex == 255)
    return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
  const int e2 = ex + 896 + sc;
  if (e2 <= 0) return __longlong_as_double((long long)sgn);
  if (e2 >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)e2 << 52) |
                                          ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// The same for a cell whose scale keeps every result in the double range
// (|sc| <= 896, k = (896 + sc) << 20): the exponent is rebased on the high word
// by one integer addition; zero and subnormal floats give a signed zero,
// inf and NaN stay inf and NaN.
__device__ __forceinline__ double fx_f2d_fast(float f, unsigned k) {
  const unsigned u = __float_as_uint(f);
  const unsigned a = u & 0x7FFFFFFFu, sgn = u & 0x80000000u;
  unsigned hi = ((a >> 3) + k) | sgn;
  unsigned lo = u << 29;
  if (a < 0x00800000u) hi = sgn, lo = 0u;
  if (a >= 0x7F800000u) hi = sgn | 0x7FF00000u | ((a & 0x7FFFFFu) >> 3);
  return __hiloint2double((int)hi, (int)lo);
}

// a float pair from shared memory, kept at its place in the batch loop (the
// compiler would otherwise hoist loop-invariant rows of D into registers for
// the whole kernel)
__device__ __forceinline__ float2 lds_pair(const float2 *p) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
               : "=f"(v.x), "=f"(v.y)
               : "r"((unsigned)__cvta_generic_to_shared(p)));
  return v;
}

// the scale offset of a cell from its largest biased exponent
__device__ __forceinline__ int fx_offset(int emax) { return emax > 0 ? emax - 1022 : 0; }

// Column kernel (thread (e, j, k) owns the i-column of cell e) with the bulk-TMA
// pipeline of bk5_tma_kernel: per batch, barrier A waits for G(b) (the u(b)
// gather was prefetched into registers during batch b-1, its largest exponent
// per cell reduced into s_emax by shared atomics), then the scaled u goes to
// shared memory (barrier B), map(b+next) is requested, gradient + metric run
// (barrier C), G(b+next) is requested, u(b+next) is prefetched and the
// transpose + atomic scatter of batch b runs.  MAPTMA = false loads the dof map
// with plain loads (a map array that is not 16-byte aligned).  gexp[cell] is
// the per-cell exponent offset of the scaled G.
// EXPIRE (test hook): the first G copy is armed but not issued, and every wait
// gives up after 1 ms, so the timeout path runs with no copy in flight.
template <int N, int E, int MB, bool MAPTMA, bool EXPIRE = false>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5fx_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                     const float2 *__restrict__ G, const int *__restrict__ gexp,
                     const double *__restrict__ src, double *__restrict__ dst,
                     const BasisFX<N> basis, const int *__restrict__ done_flag,
                     int *__restrict__ err_flag) {
  if (done_flag != nullptr && *done_flag) return;
  using L = TmaLayout<N, E, ArithDF>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  float2 *sG = reinterpret_cast<float2 *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  df *s_u = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  df *s_vs = s_u + E * N3;
  df *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;
  __shared__ int s_emax[2][E];

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  // D as (hi, lo) pairs: the rows and columns this thread needs with a runtime
  // index are read from here at the start of the phase that uses them, so only
  // one phase's 4N of them are live at a time
  __shared__ float2 s_D[N * N];
  for (int t = tid; t < N * N; t += blockDim.x) s_D[t] = make_float2(basis.Dh[t], basis.Dl[t]);
  const float cgj = basis.cg[j], cgk = basis.cg[k], cij = basis.ci[j], cik = basis.ci[k];

  TmaTiles<N, E, ArithDF> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  T.map_ok = MAPTMA;
  constexpr uint64_t wlim = EXPIRE ? 1000000ull : MFGB_WAIT_LIMIT_NS;
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg, wlim);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm, wlim);
  };

  if (tid < 2 * E) (&s_emax[0][0])[tid] = 0;
  if (tid == 0) {
    mbar_init(mbar_g, 1);
    mbar_init(mbar_m, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    if (EXPIRE)
      mbar_arrive_expect_tx(mbar_g, 16u);
    else
      T.issue_g(batch);
    T.issue_map(batch);
  }
  uint32_t ph_g = 0, ph_m = 0;
  uint32_t idx[N];
  double raw[N];
  int ge = 0;  // G exponent offset of this thread's cell in the prefetched batch
  // gathered column -> its largest exponent into the cell's slot
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) em = max(em, idx[i] != MFGB_INVALID_DOF ? dexp(raw[i]) : 0);
    if (em) atomicMax(&s_emax[slot][el], em);
  };
  {
    const bool ok = mbar_wait(mbar_m, ph_m, wlim);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw);
    reduce_exp(0);
    if (el < T.cells_of(batch)) ge = __ldg(gexp + batch * E + el);
  }

  for (int it = 0; batch < n_batches; batch += gridDim.x, ++it) {
    const int slot = it & 1;
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g, wlim);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase by barrier B
    const int su = fx_offset(s_emax[slot][el]);
    const int sc = su + ge;  // the cell's result scale
    const bool fast_out = (unsigned)(sc + 896) <= 1792u;
    const unsigned kout = (unsigned)(896 + sc) << 20;
    df u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = idx[i] != MFGB_INVALID_DOF ? fx_from_double(raw[i], su) : df{0.f, 0.f};
      s_u[el * N3 + i * N2 + jk] = u[i];
    }
    __syncthreads();  // barrier B: s_u ready, s_emax[slot] read; the map tile is free
    if (jk == 0) s_emax[slot][el] = 0;  // next written after barrier C of the next batch
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }

    const bool valid = el < T.cells_of(batch);
    float Djh[N], Djl[N], Dkh[N], Dkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + j * N + m), b = lds_pair(s_D + k * N + m);
      Djh[m] = a.x, Djl[m] = a.y, Dkh[m] = b.x, Dkl[m] = b.y;
    }
    df vr[N];
    const float2 *Gc = sG + el * 6 * N3 + jk;
#pragma unroll
    for (int i = 0; i < N; ++i) {
      // ---- gradient: q_r = D[i][.] u(., j, k), q_s = D[j][.] u(i, ., k), q_t = D[k][.] u(i, j, .)
      fxacc ar, as, at;
      const float cr = basis.cg[i];
      fx_first(ar, basis.Dh[i * N], basis.Dl[i * N], u[0].hi, u[0].lo, cr);
      {
        const df a = s_u[el * N3 + i * N2 + k], b = s_u[el * N3 + i * N2 + j * N];
        fx_first(as, Djh[0], Djl[0], a.hi, a.lo, cgj);
        fx_first(at, Dkh[0], Dkl[0], b.hi, b.lo, cgk);
      }
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(ar, basis.Dh[i * N + m], basis.Dl[i * N + m], u[m].hi, u[m].lo);
        const df a = s_u[el * N3 + i * N2 + m * N + k], b = s_u[el * N3 + i * N2 + j * N + m];
        fx_fma(as, Djh[m], Djl[m], a.hi, a.lo);
        fx_fma(at, Dkh[m], Dkl[m], b.hi, b.lo);
      }
      const df qr = fx_finish(ar, cr), qs = fx_finish(as, cgj), qt = fx_finish(at, cgk);
      // ---- metric, bound per point: max |q| times the row sums of |G|
      float2 grr = make_float2(0.f, 0.f), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = Gc[0 * N3 + i * N2];
        grs = Gc[1 * N3 + i * N2];
        grt = Gc[2 * N3 + i * N2];
        gss = Gc[3 * N3 + i * N2];
        gst = Gc[4 * N3 + i * N2];
        gtt = Gc[5 * N3 + i * N2];
      }
      const float kq = basis.K * fmaxf(fmaxf(fabsf(qr.hi), fabsf(qs.hi)), fabsf(qt.hi));
      const float Cr = (fabsf(grr.x) + fabsf(grs.x) + fabsf(grt.x)) * kq;
      const float Cs = (fabsf(grs.x) + fabsf(gss.x) + fabsf(gst.x)) * kq;
      const float Ct = (fabsf(grt.x) + fabsf(gst.x) + fabsf(gtt.x)) * kq;
      fxacc br, bs, bt;
      fx_first(br, grr.x, grr.y, qr.hi, qr.lo, Cr);
      fx_fma(br, grs.x, grs.y, qs.hi, qs.lo);
      fx_fma(br, grt.x, grt.y, qt.hi, qt.lo);
      fx_first(bs, grs.x, grs.y, qr.hi, qr.lo, Cs);
      fx_fma(bs, gss.x, gss.y, qs.hi, qs.lo);
      fx_fma(bs, gst.x, gst.y, qt.hi, qt.lo);
      fx_first(bt, grt.x, grt.y, qr.hi, qr.lo, Ct);
      fx_fma(bt, gst.x, gst.y, qs.hi, qs.lo);
      fx_fma(bt, gtt.x, gtt.y, qt.hi, qt.lo);
      vr[i] = fx_finish(br, Cr);
      s_vs[el * N3 + i * N2 + jk] = fx_finish(bs, Cs);
      s_vt[el * N3 + i * N2 + jk] = fx_finish(bt, Ct);
    }
    __syncthreads();  // barrier C: G tile consumed, s_vs / s_vt ready
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }

    // this batch's scatter targets; then prefetch the next batch's gather
    uint32_t cur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cur[i] = idx[i];
    if (has_next) {
      const bool okm = mbar_wait(mbar_m, ph_m, wlim);
      if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
      ph_m ^= 1u;
      if (okm) {
        T.gather(next, el, jk, idx, raw);
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = 0.0; }
      }
      ge = el < T.cells_of(next) ? __ldg(gexp + next * E + el) : 0;
    }

    // ---- transpose: y = sum_m D[m][i] v_r(m,j,k) + D[m][j] v_s(i,m,k) + D[m][k] v_t(i,j,m);
    // the bound of output i: max |v_r| of the own column and the maxima of the
    // s- and t-lines it reads
    float Dtjh[N], Dtjl[N], Dtkh[N], Dtkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + m * N + j), b = lds_pair(s_D + m * N + k);
      Dtjh[m] = a.x, Dtjl[m] = a.y, Dtkh[m] = b.x, Dtkl[m] = b.y;
    }
    float mr = 0.f;
#pragma unroll
    for (int m = 0; m < N; ++m) mr = fmaxf(mr, fabsf(vr[m].hi));
#pragma unroll
    for (int i = 0; i < N; ++i) {
      df ls[N], lt[N];
      float ms = 0.f, mt = 0.f;
#pragma unroll
      for (int m = 0; m < N; ++m) {
        ls[m] = s_vs[el * N3 + i * N2 + m * N + k];
        lt[m] = s_vt[el * N3 + i * N2 + j * N + m];
        ms = fmaxf(ms, fabsf(ls[m].hi));
        mt = fmaxf(mt, fabsf(lt[m].hi));
      }
      const float C = __fmaf_rn(mt, cik, __fmaf_rn(ms, cij, mr * basis.ci[i]));
      fxacc a;
      fx_first(a, basis.Dh[i], basis.Dl[i], vr[0].hi, vr[0].lo, C);
      fx_fma(a, Dtjh[0], Dtjl[0], ls[0].hi, ls[0].lo);
      fx_fma(a, Dtkh[0], Dtkl[0], lt[0].hi, lt[0].lo);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(a, basis.Dh[m * N + i], basis.Dl[m * N + i], vr[m].hi, vr[m].lo);
        fx_fma(a, Dtjh[m], Dtjl[m], ls[m].hi, ls[m].lo);
        fx_fma(a, Dtkh[m], Dtkl[m], lt[m].hi, lt[m].lo);
      }
      const df y = fx_finish(a, C);
      if (cur[i] != MFGB_INVALID_DOF)
        atomicAdd(dst + cur[i], fast_out ? fx_f2d_fast(y.hi, kout) + fx_f2d_fast(y.lo, kout)
                                         : fx_f2d(y.hi, sc) + fx_f2d(y.lo, sc));
    }
    // the prefetched gather's largest exponent per cell, once its loads have
    // landed (read after the next barrier A)
    if (has_next) reduce_exp(slot ^ 1);
  }
}


// BK6 (NC interleaved components per node sharing one G tile) with the offset
// accumulation and per-cell scaling of the kernel above: per batch the scaled
// G pairs arrive once, and the components run one after another, each with its
// own exponent offset per cell (reduced while the previous component
// integrates, read after one extra barrier).  The next component's gather is
// prefetched during the current component's transpose, the next batch's first
// component during the last one.
template <int N, int E, int MB, bool MAPTMA, int NC>
__global__ void __launch_bounds__(E * N * N, MB)
    bk6fx_tma_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                     const float2 *__restrict__ G, const int *__restrict__ gexp,
                     const double *__restrict__ src, double *__restrict__ dst,
                     const BasisFX<N> basis, int *__restrict__ err_flag) {
  using L = TmaLayout<N, E, ArithDF>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  float2 *sG = reinterpret_cast<float2 *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  df *s_u = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  df *s_vs = s_u + E * N3;
  df *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;
  __shared__ int s_emax[2][E];

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  __shared__ float2 s_D[N * N];
  for (int t = tid; t < N * N; t += blockDim.x) s_D[t] = make_float2(basis.Dh[t], basis.Dl[t]);
  const float cgj = basis.cg[j], cgk = basis.cg[k], cij = basis.ci[j], cik = basis.ci[k];

  TmaTiles<N, E, ArithDF> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  T.map_ok = MAPTMA;
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm);
  };

  if (tid < 2 * E) (&s_emax[0][0])[tid] = 0;
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
  double raw[N];
  int ge = 0;  // G exponent offset of this thread's cell in the prefetched batch
  // dof indices of column (el, jk) of batch b, from the map tile or global
  auto indices = [&](int64_t b) {
    const int cells = T.cells_of(b);
    const bool ok = el < cells;
    const bool mt = T.map_by_tma(cells);
#pragma unroll
    for (int i = 0; i < N; ++i)
      idx[i] = ok ? (mt ? sMap[el * N3 + i * N2 + jk] : __ldg(map + (b * E + el) * N3 + i * N2 + jk))
                  : MFGB_INVALID_DOF;
  };
  auto gather = [&](int c) {
#pragma unroll
    for (int i = 0; i < N; ++i)
      raw[i] = idx[i] != MFGB_INVALID_DOF ? __ldg(src + (size_t)NC * idx[i] + c) : 0.0;
  };
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) em = max(em, idx[i] != MFGB_INVALID_DOF ? dexp(raw[i]) : 0);
    if (em) atomicMax(&s_emax[slot][el], em);
  };
  {
    const bool ok = mbar_wait(mbar_m, ph_m);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    indices(batch);
    gather(0);
    reduce_exp(0);
    if (el < T.cells_of(batch)) ge = __ldg(gexp + batch * E + el);
  }

  int cnt = 0;  // components run so far: the exponent slot alternates with it
  for (; batch < n_batches; batch += gridDim.x) {
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase by barrier B
    const bool valid = el < T.cells_of(batch);
    const float2 *Gc = sG + el * 6 * N3 + jk;
    const int ge_batch = ge;
#pragma unroll 1
    for (int c = 0; c < NC; ++c, ++cnt) {
      const int slot = cnt & 1;
      if (c > 0) __syncthreads();  // this component's exponents are in; s_u is free
      const int su = fx_offset(s_emax[slot][el]);
      const int sc = su + ge_batch;  // the cell's result scale for this component
      const bool fast_out = (unsigned)(sc + 896) <= 1792u;
      const unsigned kout = (unsigned)(896 + sc) << 20;
      df u[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        u[i] = idx[i] != MFGB_INVALID_DOF ? fx_from_double(raw[i], su) : df{0.f, 0.f};
        s_u[el * N3 + i * N2 + jk] = u[i];
      }
      __syncthreads();  // barrier B: s_u ready, s_emax[slot] read (c = 0: the map tile is free)
      if (jk == 0) s_emax[slot][el] = 0;  // next written two components on
      if (c == 0 && tid == 0 && has_next) {
        fence_proxy_async_smem();
        T.issue_map(next);
      }
      float Djh[N], Djl[N], Dkh[N], Dkl[N];
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const float2 a = lds_pair(s_D + j * N + m), b = lds_pair(s_D + k * N + m);
        Djh[m] = a.x, Djl[m] = a.y, Dkh[m] = b.x, Dkl[m] = b.y;
      }
      df vr[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        fxacc ar, as, at;
        const float cr = basis.cg[i];
        fx_first(ar, basis.Dh[i * N], basis.Dl[i * N], u[0].hi, u[0].lo, cr);
        {
          const df a = s_u[el * N3 + i * N2 + k], b = s_u[el * N3 + i * N2 + j * N];
          fx_first(as, Djh[0], Djl[0], a.hi, a.lo, cgj);
          fx_first(at, Dkh[0], Dkl[0], b.hi, b.lo, cgk);
        }
#pragma unroll
        for (int m = 1; m < N; ++m) {
          fx_fma(ar, basis.Dh[i * N + m], basis.Dl[i * N + m], u[m].hi, u[m].lo);
          const df a = s_u[el * N3 + i * N2 + m * N + k], b = s_u[el * N3 + i * N2 + j * N + m];
          fx_fma(as, Djh[m], Djl[m], a.hi, a.lo);
          fx_fma(at, Dkh[m], Dkl[m], b.hi, b.lo);
        }
        const df qr = fx_finish(ar, cr), qs = fx_finish(as, cgj), qt = fx_finish(at, cgk);
        float2 grr = make_float2(0.f, 0.f), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
        if (valid) {
          grr = Gc[0 * N3 + i * N2];
          grs = Gc[1 * N3 + i * N2];
          grt = Gc[2 * N3 + i * N2];
          gss = Gc[3 * N3 + i * N2];
          gst = Gc[4 * N3 + i * N2];
          gtt = Gc[5 * N3 + i * N2];
        }
        const float kq = basis.K * fmaxf(fmaxf(fabsf(qr.hi), fabsf(qs.hi)), fabsf(qt.hi));
        const float Cr = (fabsf(grr.x) + fabsf(grs.x) + fabsf(grt.x)) * kq;
        const float Cs = (fabsf(grs.x) + fabsf(gss.x) + fabsf(gst.x)) * kq;
        const float Ct = (fabsf(grt.x) + fabsf(gst.x) + fabsf(gtt.x)) * kq;
        fxacc br, bs, bt;
        fx_first(br, grr.x, grr.y, qr.hi, qr.lo, Cr);
        fx_fma(br, grs.x, grs.y, qs.hi, qs.lo);
        fx_fma(br, grt.x, grt.y, qt.hi, qt.lo);
        fx_first(bs, grs.x, grs.y, qr.hi, qr.lo, Cs);
        fx_fma(bs, gss.x, gss.y, qs.hi, qs.lo);
        fx_fma(bs, gst.x, gst.y, qt.hi, qt.lo);
        fx_first(bt, grt.x, grt.y, qr.hi, qr.lo, Ct);
        fx_fma(bt, gst.x, gst.y, qs.hi, qs.lo);
        fx_fma(bt, gtt.x, gtt.y, qt.hi, qt.lo);
        vr[i] = fx_finish(br, Cr);
        s_vs[el * N3 + i * N2 + jk] = fx_finish(bs, Cs);
        s_vt[el * N3 + i * N2 + jk] = fx_finish(bt, Ct);
      }
      __syncthreads();  // barrier C: s_vs / s_vt ready (last component: G tile consumed)
      if (c == NC - 1 && tid == 0 && has_next) {
        fence_proxy_async_smem();
        T.issue_g(next);
      }
      // this component's scatter targets; then prefetch the next component
      // (the next batch's first one after the last)
      uint32_t cur[N];
#pragma unroll
      for (int i = 0; i < N; ++i) cur[i] = idx[i];
      if (c + 1 < NC) {
        gather(c + 1);
      } else if (has_next) {
        const bool okm = mbar_wait(mbar_m, ph_m);
        if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
        ph_m ^= 1u;
        if (okm) {
          indices(next);
          gather(0);
        } else {
#pragma unroll
          for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = 0.0; }
        }
        ge = el < T.cells_of(next) ? __ldg(gexp + next * E + el) : 0;
      }
      float Dtjh[N], Dtjl[N], Dtkh[N], Dtkl[N];
#pragma unroll
      for (int m = 0; m < N; ++m) {
        const float2 a = lds_pair(s_D + m * N + j), b = lds_pair(s_D + m * N + k);
        Dtjh[m] = a.x, Dtjl[m] = a.y, Dtkh[m] = b.x, Dtkl[m] = b.y;
      }
      float mr = 0.f;
#pragma unroll
      for (int m = 0; m < N; ++m) mr = fmaxf(mr, fabsf(vr[m].hi));
#pragma unroll
      for (int i = 0; i < N; ++i) {
        df ls[N], lt[N];
        float ms = 0.f, mt = 0.f;
#pragma unroll
        for (int m = 0; m < N; ++m) {
          ls[m] = s_vs[el * N3 + i * N2 + m * N + k];
          lt[m] = s_vt[el * N3 + i * N2 + j * N + m];
          ms = fmaxf(ms, fabsf(ls[m].hi));
          mt = fmaxf(mt, fabsf(lt[m].hi));
        }
        const float C = __fmaf_rn(mt, cik, __fmaf_rn(ms, cij, mr * basis.ci[i]));
        fxacc a;
        fx_first(a, basis.Dh[i], basis.Dl[i], vr[0].hi, vr[0].lo, C);
        fx_fma(a, Dtjh[0], Dtjl[0], ls[0].hi, ls[0].lo);
        fx_fma(a, Dtkh[0], Dtkl[0], lt[0].hi, lt[0].lo);
#pragma unroll
        for (int m = 1; m < N; ++m) {
          fx_fma(a, basis.Dh[m * N + i], basis.Dl[m * N + i], vr[m].hi, vr[m].lo);
          fx_fma(a, Dtjh[m], Dtjl[m], ls[m].hi, ls[m].lo);
          fx_fma(a, Dtkh[m], Dtkl[m], lt[m].hi, lt[m].lo);
        }
        const df y = fx_finish(a, C);
        if (cur[i] != MFGB_INVALID_DOF)
          atomicAdd(dst + (size_t)NC * cur[i] + c,
                    fast_out ? fx_f2d_fast(y.hi, kout) + fx_f2d_fast(y.lo, kout)
                             : fx_f2d(y.hi, sc) + fx_f2d(y.lo, sc));
      }
      // the prefetched component's largest exponent per cell (read after the
      // next component's first barrier, or the next batch's barrier A)
      if (c + 1 < NC || has_next) reduce_exp(slot ^ 1);
    }
  }
}

// The same kernel on the caller's FP64 G (the BK5 L-vector seam, deal.II's
// MatrixFree kernel, bakeoff_problems_dealii/include/bk3_kokkos_kernel.h):
// G[cell][6][n^3] arrives by bulk copies, each cell's largest G exponent is
// reduced in shared memory and the metric converts G to pairs scaled by it as
// it reads them.  Any input range is carried.
template <int N, int E, int MB, bool MAPTMA>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5fx_g64_kernel(const int64_t n_cells, const uint32_t *__restrict__ map,
                     const double *__restrict__ G, const double *__restrict__ src,
                     double *__restrict__ dst, const BasisFX<N> basis,
                     int *__restrict__ err_flag) {
  using L = TmaLayout<N, E, ArithF64>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  double *sG = reinterpret_cast<double *>(smem);
  uint32_t *sMap = reinterpret_cast<uint32_t *>(smem + L::g_bytes);
  df *s_u = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  df *s_vs = s_u + E * N3;
  df *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar, *mbar_m = mbar + 1;
  __shared__ int s_emax[2][E];
  __shared__ int s_gmax[E];  // largest biased exponent of the cell's G

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  // D as (hi, lo) pairs: the rows and columns this thread needs with a runtime
  // index are read from here at the start of the phase that uses them, so only
  // one phase's 4N of them are live at a time
  __shared__ float2 s_D[N * N];
  for (int t = tid; t < N * N; t += blockDim.x) s_D[t] = make_float2(basis.Dh[t], basis.Dl[t]);
  const float cgj = basis.cg[j], cgk = basis.cg[k], cij = basis.ci[j], cik = basis.ci[k];

  TmaTiles<N, E, ArithF64> T{n_cells, map, G, src, sG, sMap, mbar_g, mbar_m};
  T.map_ok = MAPTMA;
  constexpr uint64_t wlim = MFGB_WAIT_LIMIT_NS;
  auto fail = [&](uint32_t pg, uint32_t pm) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg, wlim);  // bounded waits for copies still in flight
    mbar_wait(mbar_m, pm, wlim);
  };

  if (tid < 2 * E) (&s_emax[0][0])[tid] = 0;
  if (tid < E) s_gmax[tid] = 0;
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
  double raw[N];
  // gathered column -> its largest exponent into the cell's slot
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) em = max(em, idx[i] != MFGB_INVALID_DOF ? dexp(raw[i]) : 0);
    if (em) atomicMax(&s_emax[slot][el], em);
  };
  {
    const bool ok = mbar_wait(mbar_m, ph_m, wlim);
    if (__syncthreads_or(!ok)) { fail(ph_g, ph_m); return; }
    ph_m ^= 1u;
    T.gather(batch, el, jk, idx, raw);
    reduce_exp(0);
  }

  for (int it = 0; batch < n_batches; batch += gridDim.x, ++it) {
    const int slot = it & 1;
    const int64_t next = batch + gridDim.x;
    const bool has_next = next < n_batches;
    const bool okg = mbar_wait(mbar_g, ph_g, wlim);
    if (__syncthreads_or(!okg)) { fail(ph_g, ph_m); return; }  // barrier A
    ph_g ^= 1u;
    T.load_g_plain(batch, tid, blockDim.x);  // ordered before the metric phase by barrier B
    const double *Gd = sG + el * 6 * N3 + jk;
    if (el < T.cells_of(batch)) {  // the cell's largest G exponent (read after barrier B)
      int eg = 0;
#pragma unroll 1
      for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int i = 0; i < N; ++i) eg = max(eg, dexp(Gd[c * N3 + i * N2]));
      if (eg) atomicMax(&s_gmax[el], eg);
    }
    const int su = fx_offset(s_emax[slot][el]);
    df u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = idx[i] != MFGB_INVALID_DOF ? fx_from_double(raw[i], su) : df{0.f, 0.f};
      s_u[el * N3 + i * N2 + jk] = u[i];
    }
    __syncthreads();  // barrier B: s_u and s_gmax ready, s_emax[slot] read; the map tile is free
    if (jk == 0) s_emax[slot][el] = 0;  // next written after barrier C of the next batch
    const int sg = fx_offset(s_gmax[el]);
    const int sc = su + sg;  // the cell's result scale
    const bool fast_out = (unsigned)(sc + 896) <= 1792u;
    const unsigned kout = (unsigned)(896 + sc) << 20;
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_map(next);
    }

    const bool valid = el < T.cells_of(batch);
    float Djh[N], Djl[N], Dkh[N], Dkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + j * N + m), b = lds_pair(s_D + k * N + m);
      Djh[m] = a.x, Djl[m] = a.y, Dkh[m] = b.x, Dkl[m] = b.y;
    }
    df vr[N];
    // G converted to pairs scaled by 2^-sg as it is read
    auto gpair = [&](int c, int i) {
      const df d = fx_from_double(Gd[c * N3 + i * N2], sg);
      return make_float2(d.hi, d.lo);
    };
#pragma unroll
    for (int i = 0; i < N; ++i) {
      // ---- gradient: q_r = D[i][.] u(., j, k), q_s = D[j][.] u(i, ., k), q_t = D[k][.] u(i, j, .)
      fxacc ar, as, at;
      const float cr = basis.cg[i];
      fx_first(ar, basis.Dh[i * N], basis.Dl[i * N], u[0].hi, u[0].lo, cr);
      {
        const df a = s_u[el * N3 + i * N2 + k], b = s_u[el * N3 + i * N2 + j * N];
        fx_first(as, Djh[0], Djl[0], a.hi, a.lo, cgj);
        fx_first(at, Dkh[0], Dkl[0], b.hi, b.lo, cgk);
      }
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(ar, basis.Dh[i * N + m], basis.Dl[i * N + m], u[m].hi, u[m].lo);
        const df a = s_u[el * N3 + i * N2 + m * N + k], b = s_u[el * N3 + i * N2 + j * N + m];
        fx_fma(as, Djh[m], Djl[m], a.hi, a.lo);
        fx_fma(at, Dkh[m], Dkl[m], b.hi, b.lo);
      }
      const df qr = fx_finish(ar, cr), qs = fx_finish(as, cgj), qt = fx_finish(at, cgk);
      // ---- metric, bound per point: max |q| times the row sums of |G|
      float2 grr = make_float2(0.f, 0.f), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = gpair(0, i);
        grs = gpair(1, i);
        grt = gpair(2, i);
        gss = gpair(3, i);
        gst = gpair(4, i);
        gtt = gpair(5, i);
      }
      const float kq = basis.K * fmaxf(fmaxf(fabsf(qr.hi), fabsf(qs.hi)), fabsf(qt.hi));
      const float Cr = (fabsf(grr.x) + fabsf(grs.x) + fabsf(grt.x)) * kq;
      const float Cs = (fabsf(grs.x) + fabsf(gss.x) + fabsf(gst.x)) * kq;
      const float Ct = (fabsf(grt.x) + fabsf(gst.x) + fabsf(gtt.x)) * kq;
      fxacc br, bs, bt;
      fx_first(br, grr.x, grr.y, qr.hi, qr.lo, Cr);
      fx_fma(br, grs.x, grs.y, qs.hi, qs.lo);
      fx_fma(br, grt.x, grt.y, qt.hi, qt.lo);
      fx_first(bs, grs.x, grs.y, qr.hi, qr.lo, Cs);
      fx_fma(bs, gss.x, gss.y, qs.hi, qs.lo);
      fx_fma(bs, gst.x, gst.y, qt.hi, qt.lo);
      fx_first(bt, grt.x, grt.y, qr.hi, qr.lo, Ct);
      fx_fma(bt, gst.x, gst.y, qs.hi, qs.lo);
      fx_fma(bt, gtt.x, gtt.y, qt.hi, qt.lo);
      vr[i] = fx_finish(br, Cr);
      s_vs[el * N3 + i * N2 + jk] = fx_finish(bs, Cs);
      s_vt[el * N3 + i * N2 + jk] = fx_finish(bt, Ct);
    }
    __syncthreads();  // barrier C: G tile consumed, s_vs / s_vt ready; s_gmax read
    if (jk == 0) s_gmax[el] = 0;
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }

    // this batch's scatter targets; then prefetch the next batch's gather
    uint32_t cur[N];
#pragma unroll
    for (int i = 0; i < N; ++i) cur[i] = idx[i];
    if (has_next) {
      const bool okm = mbar_wait(mbar_m, ph_m, wlim);
      if (!okm && err_flag) atomicOr(err_flag, 1);  // the launch's result is void
      ph_m ^= 1u;
      if (okm) {
        T.gather(next, el, jk, idx, raw);
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) { idx[i] = MFGB_INVALID_DOF; raw[i] = 0.0; }
      }
    }

    // ---- transpose: y = sum_m D[m][i] v_r(m,j,k) + D[m][j] v_s(i,m,k) + D[m][k] v_t(i,j,m);
    // the bound of output i: max |v_r| of the own column and the maxima of the
    // s- and t-lines it reads
    float Dtjh[N], Dtjl[N], Dtkh[N], Dtkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + m * N + j), b = lds_pair(s_D + m * N + k);
      Dtjh[m] = a.x, Dtjl[m] = a.y, Dtkh[m] = b.x, Dtkl[m] = b.y;
    }
    float mr = 0.f;
#pragma unroll
    for (int m = 0; m < N; ++m) mr = fmaxf(mr, fabsf(vr[m].hi));
#pragma unroll
    for (int i = 0; i < N; ++i) {
      df ls[N], lt[N];
      float ms = 0.f, mt = 0.f;
#pragma unroll
      for (int m = 0; m < N; ++m) {
        ls[m] = s_vs[el * N3 + i * N2 + m * N + k];
        lt[m] = s_vt[el * N3 + i * N2 + j * N + m];
        ms = fmaxf(ms, fabsf(ls[m].hi));
        mt = fmaxf(mt, fabsf(lt[m].hi));
      }
      const float C = __fmaf_rn(mt, cik, __fmaf_rn(ms, cij, mr * basis.ci[i]));
      fxacc a;
      fx_first(a, basis.Dh[i], basis.Dl[i], vr[0].hi, vr[0].lo, C);
      fx_fma(a, Dtjh[0], Dtjl[0], ls[0].hi, ls[0].lo);
      fx_fma(a, Dtkh[0], Dtkl[0], lt[0].hi, lt[0].lo);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(a, basis.Dh[m * N + i], basis.Dl[m * N + i], vr[m].hi, vr[m].lo);
        fx_fma(a, Dtjh[m], Dtjl[m], ls[m].hi, ls[m].lo);
        fx_fma(a, Dtkh[m], Dtkl[m], lt[m].hi, lt[m].lo);
      }
      const df y = fx_finish(a, C);
      if (cur[i] != MFGB_INVALID_DOF)
        atomicAdd(dst + cur[i], fast_out ? fx_f2d_fast(y.hi, kout) + fx_f2d_fast(y.lo, kout)
                                         : fx_f2d(y.hi, sc) + fx_f2d(y.lo, sc));
    }
    // the prefetched gather's largest exponent per cell, once its loads have
    // landed (read after the next barrier A)
    if (has_next) reduce_exp(slot ^ 1);
  }
}


// E-vector form of the kernel above (the CEED BK5 E-vector seam,
// CEED_BK/include/kernels/BK5/templated_cuda_kernels.cuh:11-14): the caller's
// FP64 G[e][6][n^3] arrives by bulk copies, each element's largest G exponent
// is reduced in shared memory, and the metric converts G to pairs scaled by it
// as it reads them; input and output are contiguous (plain loads prefetched a
// batch ahead, plain stores).  Any input range is carried.
template <int N, int E, int MB>
__global__ void __launch_bounds__(E * N * N, MB)
    bk5fx_evec_kernel(const int64_t n_cells, const double *__restrict__ G,
                      const double *__restrict__ src, double *__restrict__ dst,
                      const BasisFX<N> basis, int *__restrict__ err_flag) {
  using L = TmaLayout<N, E, ArithF64>;
  constexpr int N2 = N * N, N3 = N * N * N;
  extern __shared__ __align__(128) unsigned char smem[];
  double *sG = reinterpret_cast<double *>(smem);
  df *s_u = reinterpret_cast<df *>(smem + L::g_bytes + L::map_bytes);
  df *s_vs = s_u + E * N3;
  df *s_vt = s_vs + E * N3;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem + L::g_bytes + L::map_bytes + L::work_bytes);
  uint64_t *mbar_g = mbar;
  __shared__ int s_emax[2][E];
  __shared__ int s_gmax[E];  // largest biased exponent of the element's G

  const int tid = threadIdx.x;
  const int el = tid / N2;
  const int jk = tid - el * N2;
  const int j = jk / N;
  const int k = jk - j * N;
  const int64_t n_batches = (n_cells + E - 1) / E;
  int64_t batch = blockIdx.x;
  if (batch >= n_batches) return;  // uniform across the CTA

  // D as (hi, lo) pairs: the rows and columns this thread needs with a runtime
  // index are read from here at the start of the phase that uses them, so only
  // one phase's 4N of them are live at a time
  __shared__ float2 s_D[N * N];
  for (int t = tid; t < N * N; t += blockDim.x) s_D[t] = make_float2(basis.Dh[t], basis.Dl[t]);
  const float cgj = basis.cg[j], cgk = basis.cg[k], cij = basis.ci[j], cik = basis.ci[k];

  // the G tiles (FP64, the caller's array) by bulk copies; no dof map
  TmaTiles<N, E, ArithF64> T{n_cells, nullptr, G, src, sG, nullptr, mbar_g, nullptr};
  auto fail = [&](uint32_t pg) {
    if (tid == 0 && err_flag) atomicOr(err_flag, 1);
    mbar_wait(mbar_g, pg);  // bounded wait for the copy still in flight
  };

  if (tid < 2 * E) (&s_emax[0][0])[tid] = 0;
  if (tid < E) s_gmax[tid] = 0;
  if (tid == 0) {
    mbar_init(mbar_g, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) T.issue_g(batch);
  uint32_t ph_g = 0;
  double raw[N];
  // this thread's column of element e of batch bt (E-vector: contiguous)
  auto load = [&](int64_t bt) {
    const int64_t e = bt * E + el;
    const bool ok = e < n_cells;
#pragma unroll
    for (int i = 0; i < N; ++i) raw[i] = ok ? __ldg(src + e * N3 + i * N2 + jk) : 0.0;
  };
  auto reduce_exp = [&](int slot) {
    int em = 0;
#pragma unroll
    for (int i = 0; i < N; ++i) em = max(em, dexp(raw[i]));
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
    const double *Gd = sG + el * 6 * N3 + jk;
    if (valid) {  // the element's largest G exponent (read after barrier B)
      int eg = 0;
#pragma unroll 1
      for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int i = 0; i < N; ++i) eg = max(eg, dexp(Gd[c * N3 + i * N2]));
      if (eg) atomicMax(&s_gmax[el], eg);
    }
    const int su = fx_offset(s_emax[slot][el]);
    df u[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      u[i] = fx_from_double(raw[i], su);
      s_u[el * N3 + i * N2 + jk] = u[i];
    }
    __syncthreads();  // barrier B: s_u and s_gmax ready, s_emax[slot] read
    if (jk == 0) s_emax[slot][el] = 0;  // next written after barrier C of the next batch
    const int sg = fx_offset(s_gmax[el]);
    const int sc = su + sg;  // the element's result scale
    const bool fast_out = (unsigned)(sc + 896) <= 1792u;
    const unsigned kout = (unsigned)(896 + sc) << 20;

    float Djh[N], Djl[N], Dkh[N], Dkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + j * N + m), b = lds_pair(s_D + k * N + m);
      Djh[m] = a.x, Djl[m] = a.y, Dkh[m] = b.x, Dkl[m] = b.y;
    }
    df vr[N];
    // G converted to pairs scaled by 2^-sg as it is read
    auto gpair = [&](int c, int i) {
      const df d = fx_from_double(Gd[c * N3 + i * N2], sg);
      return make_float2(d.hi, d.lo);
    };
#pragma unroll
    for (int i = 0; i < N; ++i) {
      // ---- gradient: q_r = D[i][.] u(., j, k), q_s = D[j][.] u(i, ., k), q_t = D[k][.] u(i, j, .)
      fxacc ar, as, at;
      const float cr = basis.cg[i];
      fx_first(ar, basis.Dh[i * N], basis.Dl[i * N], u[0].hi, u[0].lo, cr);
      {
        const df a = s_u[el * N3 + i * N2 + k], b = s_u[el * N3 + i * N2 + j * N];
        fx_first(as, Djh[0], Djl[0], a.hi, a.lo, cgj);
        fx_first(at, Dkh[0], Dkl[0], b.hi, b.lo, cgk);
      }
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(ar, basis.Dh[i * N + m], basis.Dl[i * N + m], u[m].hi, u[m].lo);
        const df a = s_u[el * N3 + i * N2 + m * N + k], b = s_u[el * N3 + i * N2 + j * N + m];
        fx_fma(as, Djh[m], Djl[m], a.hi, a.lo);
        fx_fma(at, Dkh[m], Dkl[m], b.hi, b.lo);
      }
      const df qr = fx_finish(ar, cr), qs = fx_finish(as, cgj), qt = fx_finish(at, cgk);
      // ---- metric, bound per point: max |q| times the row sums of |G|
      float2 grr = make_float2(0.f, 0.f), grs = grr, grt = grr, gss = grr, gst = grr, gtt = grr;
      if (valid) {
        grr = gpair(0, i);
        grs = gpair(1, i);
        grt = gpair(2, i);
        gss = gpair(3, i);
        gst = gpair(4, i);
        gtt = gpair(5, i);
      }
      const float kq = basis.K * fmaxf(fmaxf(fabsf(qr.hi), fabsf(qs.hi)), fabsf(qt.hi));
      const float Cr = (fabsf(grr.x) + fabsf(grs.x) + fabsf(grt.x)) * kq;
      const float Cs = (fabsf(grs.x) + fabsf(gss.x) + fabsf(gst.x)) * kq;
      const float Ct = (fabsf(grt.x) + fabsf(gst.x) + fabsf(gtt.x)) * kq;
      fxacc br, bs, bt;
      fx_first(br, grr.x, grr.y, qr.hi, qr.lo, Cr);
      fx_fma(br, grs.x, grs.y, qs.hi, qs.lo);
      fx_fma(br, grt.x, grt.y, qt.hi, qt.lo);
      fx_first(bs, grs.x, grs.y, qr.hi, qr.lo, Cs);
      fx_fma(bs, gss.x, gss.y, qs.hi, qs.lo);
      fx_fma(bs, gst.x, gst.y, qt.hi, qt.lo);
      fx_first(bt, grt.x, grt.y, qr.hi, qr.lo, Ct);
      fx_fma(bt, gst.x, gst.y, qs.hi, qs.lo);
      fx_fma(bt, gtt.x, gtt.y, qt.hi, qt.lo);
      vr[i] = fx_finish(br, Cr);
      s_vs[el * N3 + i * N2 + jk] = fx_finish(bs, Cs);
      s_vt[el * N3 + i * N2 + jk] = fx_finish(bt, Ct);
    }
    __syncthreads();  // barrier C: G tile consumed, s_vs / s_vt ready; s_gmax read
    if (jk == 0) s_gmax[el] = 0;
    if (tid == 0 && has_next) {
      fence_proxy_async_smem();
      T.issue_g(next);
    }

    const int64_t e_out = batch * E + el;  // this batch's element of the thread
    if (has_next) load(next);  // the next batch's column, used after its barrier A

    // ---- transpose: y = sum_m D[m][i] v_r(m,j,k) + D[m][j] v_s(i,m,k) + D[m][k] v_t(i,j,m);
    // the bound of output i: max |v_r| of the own column and the maxima of the
    // s- and t-lines it reads
    float Dtjh[N], Dtjl[N], Dtkh[N], Dtkl[N];
#pragma unroll
    for (int m = 0; m < N; ++m) {
      const float2 a = lds_pair(s_D + m * N + j), b = lds_pair(s_D + m * N + k);
      Dtjh[m] = a.x, Dtjl[m] = a.y, Dtkh[m] = b.x, Dtkl[m] = b.y;
    }
    float mr = 0.f;
#pragma unroll
    for (int m = 0; m < N; ++m) mr = fmaxf(mr, fabsf(vr[m].hi));
#pragma unroll
    for (int i = 0; i < N; ++i) {
      df ls[N], lt[N];
      float ms = 0.f, mt = 0.f;
#pragma unroll
      for (int m = 0; m < N; ++m) {
        ls[m] = s_vs[el * N3 + i * N2 + m * N + k];
        lt[m] = s_vt[el * N3 + i * N2 + j * N + m];
        ms = fmaxf(ms, fabsf(ls[m].hi));
        mt = fmaxf(mt, fabsf(lt[m].hi));
      }
      const float C = __fmaf_rn(mt, cik, __fmaf_rn(ms, cij, mr * basis.ci[i]));
      fxacc a;
      fx_first(a, basis.Dh[i], basis.Dl[i], vr[0].hi, vr[0].lo, C);
      fx_fma(a, Dtjh[0], Dtjl[0], ls[0].hi, ls[0].lo);
      fx_fma(a, Dtkh[0], Dtkl[0], lt[0].hi, lt[0].lo);
#pragma unroll
      for (int m = 1; m < N; ++m) {
        fx_fma(a, basis.Dh[m * N + i], basis.Dl[m * N + i], vr[m].hi, vr[m].lo);
        fx_fma(a, Dtjh[m], Dtjl[m], ls[m].hi, ls[m].lo);
        fx_fma(a, Dtkh[m], Dtkl[m], lt[m].hi, lt[m].lo);
      }
      const df y = fx_finish(a, C);
      if (e_out < n_cells)
        dst[e_out * N3 + i * N2 + jk] = fast_out ? fx_f2d_fast(y.hi, kout) + fx_f2d_fast(y.lo, kout)
                                                 : fx_f2d(y.hi, sc) + fx_f2d(y.lo, sc);
    }
    // the next batch's largest exponent per element (read after its barrier A)
    if (has_next) reduce_exp(slot ^ 1);
  }
}

}  // namespace mfgb
