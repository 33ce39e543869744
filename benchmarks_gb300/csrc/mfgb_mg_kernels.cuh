// mfgb_mg_kernels.cuh -- element-wise, Chebyshev and transfer kernels shared
// by the single-problem multigrid (mfgb_mg.cu) and the batched solver
// (mfgb_batch.cu).  Internal to the library.
#pragma once
#include <algorithm>
#include <cstdint>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"

namespace mfgb {
namespace {

constexpr int T256 = 256;

inline unsigned grid1d(int64_t n) {
  const int64_t g = (n + T256 - 1) / T256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

#define GRID_STRIDE(t, n)                                                             \
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (n); \
       t += (int64_t)gridDim.x * blockDim.x)

// Start vector of the lambda_max power iterations, entry i of a level:
// 0.5 + U[0, 1) from SplitMix64 (Steele, Lea, Flood 2014) of i, so that the
// batched set-up can generate every problem's start on the GPU in parallel.
__device__ __forceinline__ double power_start_value(uint64_t i) {
  uint64_t z = (i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return 0.5 + (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_power_start(int64_t n, double *v) {
  GRID_STRIDE(t, n) v[t] = power_start_value((uint64_t)t);
}

template <class T>
__global__ void k_fill(int64_t n, T *x, T v) {
  GRID_STRIDE(t, n) x[t] = v;
}

template <class T>
__global__ void k_copy_constrained(int64_t nc, const int64_t *__restrict__ c,
                                   const T *__restrict__ src, T *__restrict__ dst) {
  GRID_STRIDE(t, nc) dst[c[t]] = src[c[t]];
}

template <class T>
__global__ void k_set_constrained(int64_t nc, const int64_t *__restrict__ c, T *__restrict__ v,
                                  T val) {
  GRID_STRIDE(t, nc) v[c[t]] = val;
}

template <class TO, class TI>
__global__ void k_convert(int64_t n, const TI *__restrict__ a, TO *__restrict__ b) {
  GRID_STRIDE(t, n) b[t] = (TO)a[t];
}

// Chebyshev first step from x0 = 0: x = d = (1/theta) Dinv b ; r = b
template <class T>
__global__ void k_cheb_first_zero(int64_t n, const T *__restrict__ b, const T *__restrict__ dinv,
                                  T *__restrict__ x, T *__restrict__ d, T *__restrict__ r,
                                  T inv_theta) {
  GRID_STRIDE(t, n) {
    const T bt = b[t];
    const T dt = inv_theta * dinv[t] * bt;
    r[t] = bt;
    d[t] = dt;
    x[t] = dt;
  }
}

// Chebyshev first step from x0: r = b - Ax (Ax in ax); d = (1/theta) Dinv r; x += d
template <class T>
__global__ void k_cheb_first(int64_t n, const T *__restrict__ b, const T *__restrict__ ax,
                             const T *__restrict__ dinv, T *__restrict__ x, T *__restrict__ d,
                             T *__restrict__ r, T inv_theta) {
  GRID_STRIDE(t, n) {
    const T rt = b[t] - ax[t];
    const T dt = inv_theta * dinv[t] * rt;
    r[t] = rt;
    d[t] = dt;
    x[t] += dt;
  }
}

// r -= A d (in ad); d = c1 d + c2 Dinv r; x += d
template <class T>
__global__ void k_cheb_step(int64_t n, const T *__restrict__ ad, const T *__restrict__ dinv,
                            T *__restrict__ x, T *__restrict__ d, T *__restrict__ r, T c1, T c2) {
  GRID_STRIDE(t, n) {
    const T rt = r[t] - ad[t];
    const T dt = c1 * d[t] + c2 * dinv[t] * rt;
    r[t] = rt;
    d[t] = dt;
    x[t] += dt;
  }
}

// r = b - ax
template <class T>
__global__ void k_residual(int64_t n, const T *__restrict__ b, const T *__restrict__ ax,
                           T *__restrict__ r) {
  GRID_STRIDE(t, n) r[t] = b[t] - ax[t];
}

template <class T>
__global__ void k_axpy(int64_t n, T a, const T *__restrict__ x, T *__restrict__ y) {
  GRID_STRIDE(t, n) y[t] += a * x[t];
}

template <class T>
__global__ void k_scale_by(int64_t n, const T *__restrict__ s, T *__restrict__ v) {
  GRID_STRIDE(t, n) v[t] *= s[t];
}

// ---- p-transfer: fine degree pf, coarse degree pc, same cells ------------
struct PTransferParams {
  float B32[81];
  double B64[81];  // B[a*(pc+1) + b] = l^c_b(x^f_a)
  int nf, nc;      // points per direction (fine, coarse)
};

template <class T>
__device__ __forceinline__ T bval(const PTransferParams &P, int idx);
template <>
__device__ __forceinline__ float bval<float>(const PTransferParams &P, int idx) {
  return P.B32[idx];
}
template <>
__device__ __forceinline__ double bval<double>(const PTransferParams &P, int idx) {
  return P.B64[idx];
}

// Sum-factorised p-transfers: one CTA per cell, three 1D passes through
// shared memory (nc^3 -> nc*nc*nf -> nc*nf*nf -> nf^3 and back).
template <class T>
__global__ void __launch_bounds__(128)
    k_p_prolongate_sf(int64_t n_cells, const uint32_t *__restrict__ map_f,
                      const uint32_t *__restrict__ map_c, const T *__restrict__ xc,
                      T *__restrict__ tf, PTransferParams P) {
  __shared__ T s0[729], s1[729];
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  for (int64_t e = blockIdx.x; e < n_cells; e += gridDim.x) {
    for (int t = threadIdx.x; t < nc3; t += blockDim.x) {
      const uint32_t dc = map_c[e * nc3 + t];
      s0[t] = dc != MFGB_INVALID_DOF ? xc[dc] : T(0);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc * nc * nf; t += blockDim.x) {  // along k: [a][b][kf]
      const int a = t / (nc * nf), b = (t / nf) % nc, kf = t % nf;
      T s = 0;
      for (int c = 0; c < nc; ++c) s += bval<T>(P, kf * nc + c) * s0[(a * nc + b) * nc + c];
      s1[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc * nf * nf; t += blockDim.x) {  // along j: [a][jf][kf]
      const int a = t / (nf * nf), jf = (t / nf) % nf, kf = t % nf;
      T s = 0;
      for (int b = 0; b < nc; ++b) s += bval<T>(P, jf * nc + b) * s1[(a * nc + b) * nf + kf];
      s0[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nf3; t += blockDim.x) {  // along i: [if][jf][kf]
      const int i = t / (nf * nf), jk = t % (nf * nf);
      const uint32_t df = map_f[e * nf3 + t];
      if (df == MFGB_INVALID_DOF) continue;
      T s = 0;
      for (int a = 0; a < nc; ++a) s += bval<T>(P, i * nc + a) * s0[a * nf * nf + jk];
      tf[df] = s;
    }
    __syncthreads();
  }
}

template <class T>
__global__ void __launch_bounds__(128)
    k_p_restrict_sf(int64_t n_cells, const uint32_t *__restrict__ map_f,
                    const uint32_t *__restrict__ map_c, const T *__restrict__ rf,
                    const T *__restrict__ inv_val_f, T *__restrict__ rc, PTransferParams P) {
  __shared__ T s0[729], s1[729];
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  for (int64_t e = blockIdx.x; e < n_cells; e += gridDim.x) {
    for (int t = threadIdx.x; t < nf3; t += blockDim.x) {
      const uint32_t df = map_f[e * nf3 + t];
      s0[t] = df != MFGB_INVALID_DOF ? rf[df] * inv_val_f[df] : T(0);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc * nf * nf; t += blockDim.x) {  // along i: [a][jf][kf]
      const int a = t / (nf * nf), jk = t % (nf * nf);
      T s = 0;
      for (int i = 0; i < nf; ++i) s += bval<T>(P, i * nc + a) * s0[i * nf * nf + jk];
      s1[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc * nc * nf; t += blockDim.x) {  // along j: [a][b][kf]
      const int a = t / (nc * nf), b = (t / nf) % nc, kf = t % nf;
      T s = 0;
      for (int j = 0; j < nf; ++j) s += bval<T>(P, j * nc + b) * s1[(a * nf + j) * nf + kf];
      s0[t] = s;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nc3; t += blockDim.x) {  // along k: [a][b][c]
      const int a = t / (nc * nc), b = (t / nc) % nc, c = t % nc;
      const uint32_t dc = map_c[e * nc3 + t];
      if (dc == MFGB_INVALID_DOF) continue;
      T s = 0;
      for (int k = 0; k < nf; ++k) s += bval<T>(P, k * nc + c) * s0[(a * nc + b) * nf + k];
      atomicAdd(rc + dc, s);
    }
    __syncthreads();
  }
}

// Column-layout p-transfers: a CTA holds E cells and thread (e, j, k) owns the
// fine column i = 0..NF-1 of cell e in registers.  Prolongation reads the
// cell's NC^3 coarse values from shared memory and writes its fine column
// (plain writes: shared fine DoFs get the same value from every cell);
// restriction forms s[a] = sum_i B[i][a] r_i in registers, then one thread per
// coarse DoF sums B[j][b] B[k][c] s[a][j][k] over the cell and adds atomically.
template <int NF> struct PtCells {
  static constexpr int value = NF <= 3 ? 16 : NF <= 5 ? 8 : NF <= 7 ? 4 : 2;
};

template <class T, int NF, int NC>
__global__ void __launch_bounds__(NF * NF * PtCells<NF>::value)
    k_p_prolongate_col(int64_t n_cells, const uint32_t *__restrict__ map_f,
                       const uint32_t *__restrict__ map_c, const T *__restrict__ xc,
                       T *__restrict__ tf, PTransferParams P) {
  constexpr int E = PtCells<NF>::value, NF2 = NF * NF, NF3 = NF2 * NF, NC3 = NC * NC * NC;
  __shared__ T sB[NF * NC];
  __shared__ T sc[E * NC3];
  const int tid = threadIdx.x, el = tid / NF2, jk = tid - el * NF2, j = jk / NF, k = jk - j * NF;
  for (int t = tid; t < NF * NC; t += blockDim.x) sB[t] = bval<T>(P, t);
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    for (int t = tid; t < E * NC3; t += blockDim.x) {
      const int64_t c = batch * E + t / NC3;
      const uint32_t d = c < n_cells ? map_c[c * NC3 + t % NC3] : MFGB_INVALID_DOF;
      sc[t] = d != MFGB_INVALID_DOF ? xc[d] : T(0);
    }
    __syncthreads();
    const int64_t cell = batch * E + el;
    if (cell < n_cells) {
      const T *x = sc + el * NC3;
      T t2[NC];
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        T acc = 0;
#pragma unroll
        for (int b = 0; b < NC; ++b) {
          T in = 0;
#pragma unroll
          for (int c = 0; c < NC; ++c) in += sB[k * NC + c] * x[(a * NC + b) * NC + c];
          acc += sB[j * NC + b] * in;
        }
        t2[a] = acc;
      }
#pragma unroll
      for (int i = 0; i < NF; ++i) {
        const uint32_t d = map_f[cell * NF3 + i * NF2 + jk];
        if (d == MFGB_INVALID_DOF) continue;
        T v = 0;
#pragma unroll
        for (int a = 0; a < NC; ++a) v += sB[i * NC + a] * t2[a];
        tf[d] = v;
      }
    }
    __syncthreads();
  }
}

template <class T, int NF, int NC>
__global__ void __launch_bounds__(NF * NF * PtCells<NF>::value)
    k_p_restrict_col(int64_t n_cells, const uint32_t *__restrict__ map_f,
                     const uint32_t *__restrict__ map_c, const T *__restrict__ rf,
                     const T *__restrict__ inv_val_f, T *__restrict__ rc, PTransferParams P) {
  constexpr int E = PtCells<NF>::value, NF2 = NF * NF, NF3 = NF2 * NF, NC3 = NC * NC * NC;
  __shared__ T sB[NF * NC];
  __shared__ T ss[E * NC * NF2];
  const int tid = threadIdx.x, el = tid / NF2, jk = tid - el * NF2;
  for (int t = tid; t < NF * NC; t += blockDim.x) sB[t] = bval<T>(P, t);
  const int64_t n_batches = (n_cells + E - 1) / E;
  for (int64_t batch = blockIdx.x; batch < n_batches; batch += gridDim.x) {
    __syncthreads();  // sB ready / previous batch's ss consumed
    const int64_t cell = batch * E + el;
    T r[NF];
#pragma unroll
    for (int i = 0; i < NF; ++i) {
      const uint32_t d = cell < n_cells ? map_f[cell * NF3 + i * NF2 + jk] : MFGB_INVALID_DOF;
      r[i] = d != MFGB_INVALID_DOF ? rf[d] * inv_val_f[d] : T(0);
    }
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      T acc = 0;
#pragma unroll
      for (int i = 0; i < NF; ++i) acc += sB[i * NC + a] * r[i];
      ss[(el * NC + a) * NF2 + jk] = acc;
    }
    __syncthreads();
    for (int t = tid; t < E * NC3; t += blockDim.x) {
      const int e2 = t / NC3, l = t - e2 * NC3;
      const int64_t c2 = batch * E + e2;
      if (c2 >= n_cells) continue;
      const uint32_t d = map_c[c2 * NC3 + l];
      if (d == MFGB_INVALID_DOF) continue;
      const int a = l / (NC * NC), b = (l / NC) % NC, c = l % NC;
      const T *sa = ss + (e2 * NC + a) * NF2;
      T acc = 0;
#pragma unroll
      for (int jj = 0; jj < NF; ++jj) {
        T in = 0;
#pragma unroll
        for (int kk = 0; kk < NF; ++kk) in += sB[kk * NC + c] * sa[jj * NF + kk];
        acc += sB[jj * NC + b] * in;
      }
      atomicAdd(rc + d, acc);
    }
  }
}

// launch helpers: the (NF, NC) pairs of the halving rule p -> max(1, p/2)
template <class T, int NF, int NC>
void p_transfer_col(bool restrict_, int64_t n_cells, const uint32_t *map_f, const uint32_t *map_c,
                    const T *x, const T *inv_val, T *y, const PTransferParams &P, cudaStream_t s) {
  constexpr int E = PtCells<NF>::value;
  const int64_t n_batches = (n_cells + E - 1) / E;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(n_batches, 152 * 8));
  if (restrict_)
    k_p_restrict_col<T, NF, NC><<<grid, E * NF * NF, 0, s>>>(n_cells, map_f, map_c, x, inv_val, y, P);
  else
    k_p_prolongate_col<T, NF, NC><<<grid, E * NF * NF, 0, s>>>(n_cells, map_f, map_c, x, y, P);
}

// y = P x (prolongation into a zeroed y) or y += R x (restriction), any (nf, nc)
template <class T>
void p_transfer(bool restrict_, int64_t n_cells, const uint32_t *map_f, const uint32_t *map_c,
                const T *x, const T *inv_val, T *y, const PTransferParams &P, cudaStream_t s) {
  if (n_cells <= 0) return;
  const int key = P.nf * 16 + P.nc;
  switch (key) {
#define MFGB_PT(NF, NC)                                                              \
  case NF * 16 + NC:                                                                 \
    p_transfer_col<T, NF, NC>(restrict_, n_cells, map_f, map_c, x, inv_val, y, P, s); \
    return;
    MFGB_PT(3, 2) MFGB_PT(4, 2) MFGB_PT(5, 3) MFGB_PT(6, 3) MFGB_PT(7, 4) MFGB_PT(8, 4)
    MFGB_PT(9, 5)
#undef MFGB_PT
    default: break;
  }
  const unsigned grid = (unsigned)std::min<int64_t>(n_cells, 152 * 16);
  if (restrict_)
    k_p_restrict_sf<T><<<grid, 128, 0, s>>>(n_cells, map_f, map_c, x, inv_val, y, P);
  else
    k_p_prolongate_sf<T><<<grid, 128, 0, s>>>(n_cells, map_f, map_c, x, y, P);
}

// ---- h-transfer between nested structured Q1 grids -----------------------
// Level nodes of an axis sit at fine mesh nodes min(k s, nf) (BoxStride); the
// coarse level (stride 2s) keeps every other node and the last one.  x fastest.
struct HGrid {
  int64_t fx, fy, fz, cx, cy, cz;  // node counts
  int nf[3];                       // cells of the uniform mesh the strides refer to
  int s;                           // stride of the fine level
};

// 1D Q1 interpolation weight of coarse node c at fine node I: an even fine
// node is coarse node I/2; an odd one lies between (I-1)/2 and (I+1)/2 at
// the fraction of their distance its position gives (1/2 unless the last
// coarse cell is narrower)
__device__ __forceinline__ double hw(int64_t I, int64_t c, int nf, int s) {
  if ((I & 1) == 0) return c == (I >> 1) ? 1.0 : 0.0;
  const int64_t L = (I - 1) >> 1;
  const int64_t A = (I - 1) * s, P = min(I * s, (int64_t)nf), B = min((I + 1) * s, (int64_t)nf);
  const double wr = (double)(P - A) / (double)(B - A);
  return c == L ? 1.0 - wr : (c == L + 1 ? wr : 0.0);
}

// x_f[t] += (P x_c)[t] for fine node t (interior nodes only)
template <class T>
__device__ __forceinline__ void h_prolongate_node(const HGrid &g, int64_t t, const T *__restrict__ xc,
                                                  T *__restrict__ xf) {
  const int64_t I = t % g.fx, J = (t / g.fx) % g.fy, K = t / (g.fx * g.fy);
  if (I == 0 || J == 0 || K == 0 || I == g.fx - 1 || J == g.fy - 1 || K == g.fz - 1) return;
  const int64_t i0 = I / 2, j0 = J / 2, k0 = K / 2;
  T acc = 0;
  for (int64_t kk = k0; kk <= k0 + (K & 1); ++kk)
    for (int64_t jj = j0; jj <= j0 + (J & 1); ++jj)
      for (int64_t ii = i0; ii <= i0 + (I & 1); ++ii) {
        const T w = (T)(hw(I, ii, g.nf[0], g.s) * hw(J, jj, g.nf[1], g.s) *
                        hw(K, kk, g.nf[2], g.s));
        acc += w * xc[ii + g.cx * (jj + g.cy * kk)];
      }
  xf[t] += acc;
}

// r_c[t] = (P^T r_f)[t] for coarse node t (boundary nodes -> 0)
template <class T>
__device__ __forceinline__ void h_restrict_node(const HGrid &g, int64_t t, const T *__restrict__ rf,
                                                T *__restrict__ rc) {
  const int64_t i = t % g.cx, j = (t / g.cx) % g.cy, k = t / (g.cx * g.cy);
  if (i == 0 || j == 0 || k == 0 || i == g.cx - 1 || j == g.cy - 1 || k == g.cz - 1) {
    rc[t] = 0;
    return;
  }
  T acc = 0;  // fine neighbours 2i-1 .. 2i+1 exist for every interior coarse node
  for (int64_t K = 2 * k - 1; K <= 2 * k + 1; ++K)
    for (int64_t J = 2 * j - 1; J <= 2 * j + 1; ++J)
      for (int64_t I = 2 * i - 1; I <= 2 * i + 1; ++I) {
        const T w = (T)(hw(I, i, g.nf[0], g.s) * hw(J, j, g.nf[1], g.s) *
                        hw(K, k, g.nf[2], g.s));
        acc += w * rf[I + g.fx * (J + g.fy * K)];
      }
  rc[t] = acc;
}

template <class T>
__global__ void k_h_prolongate_add(HGrid g, const T *__restrict__ xc, T *__restrict__ xf) {
  GRID_STRIDE(t, g.fx * g.fy * g.fz) h_prolongate_node(g, t, xc, xf);
}

template <class T>
__global__ void k_h_restrict(HGrid g, const T *__restrict__ rf, T *__restrict__ rc) {
  GRID_STRIDE(t, g.cx * g.cy * g.cz) h_restrict_node(g, t, rf, rc);
}

// ---- valence (number of cells sharing a DoF) ----------------------------
template <class T>
__global__ void k_count_valence(int64_t n, const uint32_t *__restrict__ map, T *__restrict__ val) {
  GRID_STRIDE(t, n) {
    const uint32_t d = map[t];
    if (d != MFGB_INVALID_DOF) atomicAdd(val + d, (T)1);
  }
}

template <class T>
__global__ void k_invert_pos(int64_t n, T *__restrict__ v) {
  GRID_STRIDE(t, n) v[t] = v[t] > 0 ? (T)1 / v[t] : (T)0;
}

// ---- host helpers ---------------------------------------------------------
HGrid hgrid(const mfgb_box_desc &fb, const BoxStride &fs, const mfgb_box_desc &cb) {
  return HGrid{fb.nx + 1, fb.ny + 1, fb.nz + 1, cb.nx + 1, cb.ny + 1, cb.nz + 1,
               {fs.nf[0], fs.nf[1], fs.nf[2]}, fs.s};
}

PTransferParams ptransfer(const mfgb_operator *fine, const mfgb_operator *coarse) {
  PTransferParams P{};
  P.nf = fine->n;
  P.nc = coarse->n;
  for (int a = 0; a < P.nf; ++a)
    for (int b = 0; b < P.nc; ++b) {
      const double v = lagrange_value(P.nc, coarse->gll_x, b, fine->gll_x[a]);
      P.B64[a * P.nc + b] = v;
      P.B32[a * P.nc + b] = (float)v;
    }
  return P;
}

}  // namespace
}  // namespace mfgb
