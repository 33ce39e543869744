// mfgb_common.cuh -- shared device/host helpers for the GB300 BK5/BP5 engine.
//
// Arithmetic policies used by the templated operator kernels:
//   ArithF64  native FP64 (DFMA; GB300 runs FP64 at ~1/58 of its FP32 rate)
//   ArithF32  native FP32
//   ArithDF   "double-float": every value is an unevaluated pair hi + lo of
//             floats (about 2^-47 relative precision), computed on the FP32
//             pipes with error-free transformations: TwoProduct by FMA and
//             Knuth's TwoSum (accumulation as in Ogita, Rump & Oishi,
//             "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).
//             Conversions to and from double use integer bit operations only,
//             so no FP64-pipe conversion instruction is issued.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define MFGB_INVALID_DOF 0xFFFFFFFFu

namespace mfgb {

// ---------------------------------------------------------------- df type --
struct df {
  float hi, lo;
};

// double -> (hi, lo) with integer ops: hi = x truncated to 24 significant
// bits, lo = the remaining 29 mantissa bits rounded to float.  |x| < 2^-126
// flushes to zero; |x| >= 2^128 is outside the float exponent range and is
// returned as (+-inf, 0); NaN stays NaN.  (The GLL collocation operator scales
// every cell by a power of two first, mfgb_bk5fx.cuh; the other double-float
// kernels rely on the range check of their inputs, mfgb_api.cu.)
__device__ __forceinline__ df df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned sign = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7FFu);
  df r;
  if (e <= 896) { r.hi = 0.f; r.lo = 0.f; return r; }
  if (e >= 1151) {
    const bool nan = e == 0x7FF && ((hw & 0xFFFFFu) | lw) != 0u;
    r.hi = __uint_as_float(sign | (nan ? 0x7FC00000u : 0x7F800000u));
    r.lo = 0.f;
    return r;
  }
  const unsigned hm = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
  r.hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | hm);
  const unsigned rem = lw & 0x1FFFFFFFu;
  if (rem == 0u || e < 949) {
    r.lo = 0.f;
  } else {
    const unsigned fb = __float_as_uint(__uint2float_rn(rem));
    r.lo = __uint_as_float(sign | (fb + ((unsigned)(e - 1075) << 23)));
  }
  return r;
}

// exact float -> double widening by integer ops (subnormal floats -> 0; inf
// and NaN kept)
__device__ __forceinline__ double double_from_float_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xFFu;
  if (ex == 0u) return 0.0;
  if (ex == 0xFFu)
    return __longlong_as_double((long long)(((unsigned long long)(u & 0x80000000u) << 32) |
                                            0x7FF0000000000000ull |
                                            ((unsigned long long)(u & 0x7FFFFFu) << 29)));
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(ex + 896u) << 52) |
                               ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

__device__ __forceinline__ double df_to_double(df a) {
  return double_from_float_exact(a.hi) + double_from_float_exact(a.lo);
}

// Knuth TwoSum: s + t == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &t) {
  s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}

// lazy double-float accumulator: value = s + c
struct dfacc {
  float s, c;
};

__device__ __forceinline__ void dfacc_zero(dfacc &a) { a.s = 0.f; a.c = 0.f; }

// a += x * y   (x, y double-float)
__device__ __forceinline__ void dfacc_fma(dfacc &a, df x, df y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.hi, -p);
  float s, t;
  two_sum(a.s, p, s, t);
  a.s = s;
  float c = __fadd_rn(a.c, __fadd_rn(t, e));
  c = __fmaf_rn(x.hi, y.lo, c);
  c = __fmaf_rn(x.lo, y.hi, c);
  a.c = c;
}

// a = x * y  (the first term of a sum: the same value as dfacc_zero then
// dfacc_fma, without the addition to zero)
__device__ __forceinline__ void dfacc_set(dfacc &a, df x, df y) {
  a.s = __fmul_rn(x.hi, y.hi);
  float c = __fmaf_rn(x.hi, y.hi, -a.s);
  c = __fmaf_rn(x.hi, y.lo, c);
  a.c = __fmaf_rn(x.lo, y.hi, c);
}

// a += b  (two lazy accumulators)
__device__ __forceinline__ void dfacc_merge(dfacc &a, const dfacc &b) {
  float s, t;
  two_sum(a.s, b.s, s, t);
  a.s = s;
  a.c = __fadd_rn(a.c, __fadd_rn(b.c, t));
}

// The accumulator as a value: the pair (s, c) itself, not renormalised (|c| may
// exceed half an ulp of s).  Its consumers accept that: a product uses hi*hi
// exactly and the two cross terms in float (dropping lo*lo), and the conversion
// to double adds hi and lo with one rounding.  The error stays that of the
// renormalising form: about 2^-45 of the sum of the absolute terms for the 3-
// to 15-term sums of the operator kernels (float32 restatement, measured).
__device__ __forceinline__ df dfacc_finish(const dfacc &a) {
  df r;
  r.hi = a.s;
  r.lo = a.c;
  return r;
}

// ----------------------------------------------------- arithmetic policies --
// Every policy defines:
//   V       value type carried through the contractions
//   Acc     accumulator type (zero / fma / mul = set to the first product /
//           set = start from a value)
//   GType   storage type of one geometric-factor component
//   VecT    L-vector element type
struct ArithF64 {
  using V = double;
  using Acc = double;
  using GType = double;
  using VecT = double;
  static __device__ __forceinline__ void set(Acc &a, V x) { a = x; }
  static __device__ __forceinline__ void zero(Acc &a) { a = 0.0; }
  static __device__ __forceinline__ void fma(Acc &a, V x, V y) { a = __fma_rn(x, y, a); }
  static __device__ __forceinline__ void mul(Acc &a, V x, V y) { a = __dmul_rn(x, y); }
  static __device__ __forceinline__ void merge(Acc &a, const Acc &b) { a = __dadd_rn(a, b); }
  static __device__ __forceinline__ V finish(const Acc &a) { return a; }
  static __device__ __forceinline__ V load_vec(VecT x) { return x; }
  static __device__ __forceinline__ VecT store_vec(V x) { return x; }
  static __device__ __forceinline__ V load_g(GType g) { return g; }
  static __device__ __forceinline__ V zero_v() { return 0.0; }
  static __device__ __forceinline__ double to_double(V x) { return x; }
};

struct ArithF32 {
  using V = float;
  using Acc = float;
  using GType = float;
  using VecT = float;
  static __device__ __forceinline__ void set(Acc &a, V x) { a = x; }
  static __device__ __forceinline__ void zero(Acc &a) { a = 0.f; }
  static __device__ __forceinline__ void fma(Acc &a, V x, V y) { a = __fmaf_rn(x, y, a); }
  static __device__ __forceinline__ void mul(Acc &a, V x, V y) { a = __fmul_rn(x, y); }
  static __device__ __forceinline__ void merge(Acc &a, const Acc &b) { a = __fadd_rn(a, b); }
  static __device__ __forceinline__ V finish(const Acc &a) { return a; }
  static __device__ __forceinline__ V load_vec(VecT x) { return x; }
  static __device__ __forceinline__ VecT store_vec(V x) { return x; }
  static __device__ __forceinline__ V load_g(GType g) { return g; }
  static __device__ __forceinline__ V zero_v() { return 0.f; }
  static __device__ __forceinline__ double to_double(V x) { return (double)x; }
};

struct ArithDF {
  using V = df;
  using Acc = dfacc;
  using GType = float2;  // (hi, lo)
  using VecT = double;
  static __device__ __forceinline__ void set(Acc &a, V x) { a.s = x.hi; a.c = x.lo; }
  static __device__ __forceinline__ void zero(Acc &a) { dfacc_zero(a); }
  static __device__ __forceinline__ void fma(Acc &a, V x, V y) { dfacc_fma(a, x, y); }
  static __device__ __forceinline__ void mul(Acc &a, V x, V y) { dfacc_set(a, x, y); }
  static __device__ __forceinline__ void merge(Acc &a, const Acc &b) { dfacc_merge(a, b); }
  static __device__ __forceinline__ V finish(const Acc &a) { return dfacc_finish(a); }
  static __device__ __forceinline__ V load_vec(VecT x) { return df_from_double(x); }
  static __device__ __forceinline__ VecT store_vec(V x) { return df_to_double(x); }
  static __device__ __forceinline__ V load_g(GType g) { df r; r.hi = g.x; r.lo = g.y; return r; }
  static __device__ __forceinline__ V zero_v() { df r; r.hi = 0.f; r.lo = 0.f; return r; }
  static __device__ __forceinline__ double to_double(V x) { return df_to_double(x); }
};

// ArithDF reading FP64 geometric factors (the kernel seams, where the caller
// supplies G in double): each component is split to (hi, lo) on load.
struct ArithDFG64 : ArithDF {
  using GType = double;
  static __device__ __forceinline__ V load_g(GType g) { return df_from_double(g); }
};

// 1D derivative matrix D[point*N + basis] passed by value (kernel parameter
// space, i.e. the constant bank), in the value type of the policy.
// The even-odd tables (used when `eo` is set): the collocation derivative on
// nodes symmetric about the cell centre satisfies D[N-1-i][N-1-m] = -D[i][m],
// so y = D x splits into half-size products of the even and odd parts of x,
//   P[i][m] = (M[i][m] + M[i][N-1-m]) / 2  (m < N/2; column N/2 = M[i][mid] for odd N),
//   Q[i][m] = (M[i][m] - M[i][N-1-m]) / 2,
// for the rows i < (N+1)/2 of M = D (Pg, Qg) and of M = D^T (Pt, Qt).
template <int N, class A>
struct Basis {
  typename A::V D[N * N];
  typename A::V Pg[(N + 1) / 2][N / 2 + 1], Qg[(N + 1) / 2][N / 2 + 1];
  typename A::V Pt[(N + 1) / 2][N / 2 + 1], Qt[(N + 1) / 2][N / 2 + 1];
  int eo;
};

// y = M x in even-odd form for M[N-1-i][N-1-m] = -M[i][m] (tables of Basis):
// with e_m = x_m + x_{N-1-m}, o_m = x_m - x_{N-1-m},
//   a_i = sum_m P[i][m] e_m (+ P[i][N/2] x_mid),  b_i = sum_m Q[i][m] o_m,
//   y_i = a_i + b_i,  y_{N-1-i} = b_i - a_i  (y_mid = b_mid: a_mid vanishes),
// about N^2/2 multiply-adds and 2N additions instead of N^2 multiply-adds.
// Plain arithmetics only.
template <int N, class A>
__device__ __forceinline__ void even_odd_apply(const typename A::V (&P)[(N + 1) / 2][N / 2 + 1],
                                               const typename A::V (&Q)[(N + 1) / 2][N / 2 + 1],
                                               const typename A::V (&x)[N], typename A::V (&y)[N]) {
  using V = typename A::V;
  constexpr int H = N / 2;
  V e[H > 0 ? H : 1], o[H > 0 ? H : 1];
#pragma unroll
  for (int m = 0; m < H; ++m) {
    e[m] = x[m] + x[N - 1 - m];
    o[m] = x[m] - x[N - 1 - m];
  }
#pragma unroll
  for (int i = 0; i < (N + 1) / 2; ++i) {
    typename A::Acc a, b;
    if constexpr (N % 2) A::mul(a, P[i][H], x[H]); else A::zero(a);
#pragma unroll
    for (int m = 0; m < H; ++m) A::fma(a, P[i][m], e[m]);
    A::zero(b);
#pragma unroll
    for (int m = 0; m < H; ++m) A::fma(b, Q[i][m], o[m]);
    if (N % 2 && i == H) {
      y[i] = A::finish(b);
    } else {
      y[i] = A::finish(a) + A::finish(b);
      y[N - 1 - i] = A::finish(b) - A::finish(a);
    }
  }
}

}  // namespace mfgb
