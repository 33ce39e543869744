// mfgb_mg.cu -- geometric p- and h-multigrid V-cycle as a preconditioner for
// FP64 conjugate gradients (mixed precision: FP32 V-cycle inside FP64 CG).
//
// The reference has no multigrid for this path (mg_transfer_global_coarsening.h
// is included but unused, CEED_bp/src/bp3.cc:27); this is new work following
// the standard algorithms:
//   levels     p = p_fine -> p_fine/2 -> ... -> 1 on the fine mesh, then Q1 on
//              2:1 coarsened box meshes down to a few cells per direction;
//              operators are re-discretised on every level (same deformation)
//   transfers  p: cell-wise tensor-product interpolation at the fine GLL points;
//              restriction is its transpose with fine DoFs weighted by
//              1/valence; h: Q1 interpolation on the nested structured grids
//   smoother   Chebyshev of degree k around Jacobi on [lmax/range, 1.2 lmax]
//              (Saad, Iterative Methods, alg. 12.1), lmax by power iteration
//   coarse     FP64 Jacobi-CG on the assembled coarse matrix, one CTA
//   cycle      V(k,k): pre-smooth from zero, residual, restrict, recurse,
//              prolongate-add, post-smooth
// The V-cycle runs in FP32 (precision 32) or FP64 (precision 64, operators in
// double-float arithmetic); the outer CG is always FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"

namespace mfgb {

namespace {

constexpr int T256 = 256;

unsigned grid1d(int64_t n) {
  const int64_t g = (n + T256 - 1) / T256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, 152 * 32));
}

#define GRID_STRIDE(t, n)                                                             \
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (n); \
       t += (int64_t)gridDim.x * blockDim.x)

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

// t_f[map_f] = sum_c B(i,a) B(j,b) B(k,c) x_c[map_c]  (plain writes: every cell
// computes the same value for a shared fine DoF)
template <class T>
__global__ void k_p_prolongate(int64_t n_cells, const uint32_t *__restrict__ map_f,
                               const uint32_t *__restrict__ map_c, const T *__restrict__ xc,
                               T *__restrict__ tf, PTransferParams P) {
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  GRID_STRIDE(t, n_cells * nf3) {
    const int64_t e = t / nf3;
    const int q = (int)(t - e * nf3);
    const uint32_t df = map_f[t];
    if (df == MFGB_INVALID_DOF) continue;
    const int i = q / (nf * nf), j = (q / nf) % nf, k = q % nf;
    const uint32_t *mc = map_c + e * nc3;
    T acc = 0;
    for (int a = 0; a < nc; ++a) {
      const T wa = bval<T>(P, i * nc + a);
      for (int b = 0; b < nc; ++b) {
        const T wab = wa * bval<T>(P, j * nc + b);
        for (int c = 0; c < nc; ++c) {
          const uint32_t dc = mc[a * nc * nc + b * nc + c];
          if (dc != MFGB_INVALID_DOF) acc += wab * bval<T>(P, k * nc + c) * xc[dc];
        }
      }
    }
    tf[df] = acc;
  }
}

// r_c[map_c] += sum_f B(i,a) B(j,b) B(k,c) r_f[map_f] / valence_f
template <class T>
__global__ void k_p_restrict(int64_t n_cells, const uint32_t *__restrict__ map_f,
                             const uint32_t *__restrict__ map_c, const T *__restrict__ rf,
                             const T *__restrict__ inv_val_f, T *__restrict__ rc,
                             PTransferParams P) {
  const int nf = P.nf, nc = P.nc, nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  GRID_STRIDE(t, n_cells * nc3) {
    const int64_t e = t / nc3;
    const int q = (int)(t - e * nc3);
    const uint32_t dc = map_c[t];
    if (dc == MFGB_INVALID_DOF) continue;
    const int a = q / (nc * nc), b = (q / nc) % nc, c = q % nc;
    const uint32_t *mf = map_f + e * nf3;
    T acc = 0;
    for (int i = 0; i < nf; ++i) {
      const T wa = bval<T>(P, i * nc + a);
      for (int j = 0; j < nf; ++j) {
        const T wab = wa * bval<T>(P, j * nc + b);
        for (int k = 0; k < nf; ++k) {
          const uint32_t df = mf[i * nf * nf + j * nf + k];
          if (df != MFGB_INVALID_DOF) acc += wab * bval<T>(P, k * nc + c) * rf[df] * inv_val_f[df];
        }
      }
    }
    atomicAdd(rc + dc, acc);
  }
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

// x_f += P x_c on interior fine nodes
template <class T>
__global__ void k_h_prolongate_add(HGrid g, const T *__restrict__ xc, T *__restrict__ xf) {
  GRID_STRIDE(t, g.fx * g.fy * g.fz) {
    const int64_t I = t % g.fx, J = (t / g.fx) % g.fy, K = t / (g.fx * g.fy);
    if (I == 0 || J == 0 || K == 0 || I == g.fx - 1 || J == g.fy - 1 || K == g.fz - 1) continue;
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
}

// r_c = P^T r_f on interior coarse nodes (boundary nodes -> 0)
template <class T>
__global__ void k_h_restrict(HGrid g, const T *__restrict__ rf, T *__restrict__ rc) {
  GRID_STRIDE(t, g.cx * g.cy * g.cz) {
    const int64_t i = t % g.cx, j = (t / g.cx) % g.cy, k = t / (g.cx * g.cy);
    if (i == 0 || j == 0 || k == 0 || i == g.cx - 1 || j == g.cy - 1 || k == g.cz - 1) {
      rc[t] = 0;
      continue;
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

// ---- coarse solve: FP64 Jacobi-CG on a dense SPD matrix, one CTA ---------
// A[n][n] row-major over the n interior coarse DoFs; x = A^{-1} b to a
// relative residual of tol (max_it iterations at most).
__global__ void __launch_bounds__(T256)
    k_coarse_cg(int n, const double *__restrict__ A, const double *__restrict__ dinv,
                const int64_t *__restrict__ ids, const void *__restrict__ bsrc, int b_is_float,
                void *__restrict__ xdst, int x_is_float, double tol, int max_it,
                double *__restrict__ work) {
  double *r = work, *p = work + n, *q = work + 2 * n, *x = work + 3 * n;
  __shared__ double sh[T256 / 32 + 1];
  auto bsum = [&](double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < T256 / 32; ++w) s += sh[w];
      sh[T256 / 32] = s;
    }
    __syncthreads();
    return sh[T256 / 32];
  };
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double bi = b_is_float ? (double)((const float *)bsrc)[ids[i]]
                                 : ((const double *)bsrc)[ids[i]];
    r[i] = bi;
    x[i] = 0.0;
    p[i] = dinv[i] * bi;
  }
  __syncthreads();
  double rz = 0, rr0 = 0;
  {
    double a = 0, c = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      a += r[i] * dinv[i] * r[i];
      c += r[i] * r[i];
    }
    rz = bsum(a);
    rr0 = bsum(c);
  }
  const double target = tol * tol * rr0;
  for (int it = 0; it < max_it && rr0 > 0; ++it) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      double s = 0;
      for (int j = 0; j < n; ++j) s += A[(size_t)i * n + j] * p[j];
      q[i] = s;
    }
    __syncthreads();
    double pq = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) pq += p[i] * q[i];
    pq = bsum(pq);
    const double alpha = rz / pq;
    double rr = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      rr += r[i] * r[i];
    }
    rr = bsum(rr);
    if (rr <= target) break;
    double rzn = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) rzn += r[i] * dinv[i] * r[i];
    rzn = bsum(rzn);
    const double beta = rzn / rz;
    rz = rzn;
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = dinv[i] * r[i] + beta * p[i];
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (x_is_float)
      ((float *)xdst)[ids[i]] = (float)x[i];
    else
      ((double *)xdst)[ids[i]] = x[i];
  }
}

// ---- outer FP64 PCG kernels ----------------------------------------------
__device__ __forceinline__ double warp_block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < T256 / 32; ++w) s += sh[w];
  return s;
}

// partial sums of a.b per CTA (deterministic order)
__global__ void __launch_bounds__(T256)
    k_dot_partials(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                   double *__restrict__ part) {
  __shared__ double sh[T256 / 32];
  double s = 0;
  GRID_STRIDE(t, n) s = fma(a[t], b[t], s);
  s = warp_block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void __launch_bounds__(T256)
    k_sum_partials(const double *__restrict__ part, int n, double *__restrict__ out) {
  __shared__ double sh[T256 / 32];
  double s = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = warp_block_sum(s, sh);
  if (threadIdx.x == 0) *out = s;
}

// x += alpha p; r -= alpha v; alpha = scal[0] / scal[1]; partial |r|^2
__global__ void __launch_bounds__(T256)
    k_pcg_update(int64_t n, double *__restrict__ x, double *__restrict__ r,
                 const double *__restrict__ p, const double *__restrict__ v,
                 const double *__restrict__ scal, double *__restrict__ part) {
  __shared__ double sh[T256 / 32];
  const double alpha = scal[0] / scal[1];
  double s = 0;
  GRID_STRIDE(t, n) {
    x[t] = fma(alpha, p[t], x[t]);
    const double rt = fma(-alpha, v[t], r[t]);
    r[t] = rt;
    s = fma(rt, rt, s);
  }
  s = warp_block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// p = z + beta p, beta = scal[2] / scal[0]; then scal[0] = scal[2]  (one CTA
// updates the scalar after every CTA has read it: done by a separate kernel)
__global__ void __launch_bounds__(T256)
    k_pcg_direction(int64_t n, const double *__restrict__ z, double *__restrict__ p,
                    const double *__restrict__ scal) {
  const double beta = scal[2] / scal[0];
  GRID_STRIDE(t, n) p[t] = fma(beta, p[t], z[t]);
}

__global__ void k_copy_scalar(double *__restrict__ scal, int from, int to) {
  if (threadIdx.x == 0 && blockIdx.x == 0) scal[to] = scal[from];
}

}  // namespace

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------

struct MgLevel {
  mfgb_box_desc box{};
  BoxStride bs{};  // s = 1 on the fine mesh (p-levels), 2^l on the l-th h-level
  mfgb_operator *op = nullptr;
  int64_t n = 0;
  void *x = nullptr, *b = nullptr, *r = nullptr, *d = nullptr, *t = nullptr;
  void *inv_diag = nullptr;  // Jacobi (precision T)
  void *inv_val = nullptr;   // 1/valence (precision T), for p-restriction from this level
  double lmax = 0;
  int to_coarse = 0;  // 1 = p-transfer, 2 = h-transfer, 0 = coarsest
};

struct MgCoarse {
  int n = 0;
  double *A = nullptr, *dinv = nullptr, *work = nullptr;
  int64_t *ids = nullptr;
};

}  // namespace mfgb

struct mfgb_mg {
  int precision = 32;
  int degree = 5;
  double range = 15.0;
  double coarse_tol = 1e-12;
  std::vector<mfgb::MgLevel> levels;
  mfgb::MgCoarse coarse;
  // outer PCG buffers (FP64)
  double *r = nullptr, *z = nullptr, *p = nullptr, *v = nullptr, *part = nullptr,
         *scal = nullptr;
  int64_t outer_n = 0;
};

namespace mfgb {
namespace {

size_t tsize(int prec) { return prec == 32 ? sizeof(float) : sizeof(double); }

mfgb_status dalloc(void **p, size_t bytes) {
  *p = nullptr;
  if (!bytes) return MFGB_OK;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e, "multigrid allocation");
  }
  return MFGB_OK;
}

mfgb_status ensure_g32(mfgb_operator *op) {
  if (op->d_G32) return MFGB_OK;
  const int64_t ng = op->n_cells * 6 * (int64_t)op->n * op->n * op->n;
  mfgb_status st = dalloc((void **)&op->d_G32, sizeof(float) * ng);
  if (st) return st;
  if ((st = cuda_status(g_to_f32(ng, op->d_G, op->d_G32, nullptr), "G -> FP32"))) return st;
  return cuda_status(cudaDeviceSynchronize(), "G -> FP32");
}

// dst = A src on one level in the V-cycle precision
mfgb_status level_vmult(mfgb_operator *op, int prec, void *dst, const void *src, cudaStream_t s) {
  if (prec == 64) return vmult_impl(op, (double *)dst, (const double *)src, MFGB_ARITH_FP64_DF,
                                    nullptr, nullptr, s);
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(dst, 0, sizeof(float) * op->n_dofs, s), "A32: dst = 0")))
    return st;
  if ((st = cuda_status(bk5_f32(op->n, op->n_cells, op->d_map, op->d_G32, (const float *)src,
                                (float *)dst, op->D, nullptr, nullptr, s),
                        "A32 kernel")))
    return st;
  if (op->n_constrained)
    k_copy_constrained<float><<<grid1d(op->n_constrained), T256, 0, s>>>(
        op->n_constrained, op->d_constrained, (const float *)src, (float *)dst);
  return cuda_status(cudaGetLastError(), "A32 constrained");
}

template <class T>
mfgb_status chebyshev(const MgLevel &L, int degree, double range, bool zero_start, int prec,
                      cudaStream_t s) {
  // lambda in [lmax / range, lmax], lmax already includes the safety factor
  const double lmax = L.lmax, lmin = L.lmax / range;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  T *x = (T *)L.x, *b = (T *)L.b, *r = (T *)L.r, *d = (T *)L.d, *t = (T *)L.t;
  const T *dinv = (const T *)L.inv_diag;
  const unsigned g = grid1d(L.n);
  mfgb_status st;
  if (zero_start) {
    k_cheb_first_zero<T><<<g, T256, 0, s>>>(L.n, b, dinv, x, d, r, (T)(1.0 / theta));
  } else {
    if ((st = level_vmult(L.op, prec, t, x, s))) return st;
    k_cheb_first<T><<<g, T256, 0, s>>>(L.n, b, t, dinv, x, d, r, (T)(1.0 / theta));
  }
  for (int k = 1; k < degree; ++k) {
    if ((st = level_vmult(L.op, prec, t, d, s))) return st;
    const double rho_new = 1.0 / (2.0 * sigma - rho);
    const double c1 = rho_new * rho, c2 = 2.0 * rho_new / delta;
    k_cheb_step<T><<<g, T256, 0, s>>>(L.n, t, dinv, x, d, r, (T)c1, (T)c2);
    rho = rho_new;
  }
  return cuda_status(cudaGetLastError(), "chebyshev");
}

HGrid hgrid(const MgLevel &fine, const MgLevel &coarse) {
  return HGrid{fine.box.nx + 1, fine.box.ny + 1, fine.box.nz + 1,
               coarse.box.nx + 1, coarse.box.ny + 1, coarse.box.nz + 1,
               {fine.bs.nf[0], fine.bs.nf[1], fine.bs.nf[2]}, fine.bs.s};
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

template <class T>
mfgb_status vcycle(mfgb_mg *mg, size_t l, cudaStream_t s) {
  MgLevel &L = mg->levels[l];
  const int prec = mg->precision;
  mfgb_status st;
  if (l + 1 == mg->levels.size()) {  // coarsest: FP64 Jacobi-CG
    if ((st = cuda_status(cudaMemsetAsync(L.x, 0, sizeof(T) * L.n, s), "coarse x = 0"))) return st;
    if (mg->coarse.n > 0)
      k_coarse_cg<<<1, T256, 0, s>>>(mg->coarse.n, mg->coarse.A, mg->coarse.dinv, mg->coarse.ids,
                                     L.b, prec == 32, L.x, prec == 32, mg->coarse_tol,
                                     10 * mg->coarse.n + 100, mg->coarse.work);
    return cuda_status(cudaGetLastError(), "coarse solve");
  }
  MgLevel &C = mg->levels[l + 1];
  if ((st = chebyshev<T>(L, mg->degree, mg->range, true, prec, s))) return st;
  if ((st = level_vmult(L.op, prec, L.t, L.x, s))) return st;
  k_residual<T><<<grid1d(L.n), T256, 0, s>>>(L.n, (const T *)L.b, (const T *)L.t, (T *)L.r);
  if (L.to_coarse == 1) {
    const PTransferParams P = ptransfer(L.op, C.op);
    if ((st = cuda_status(cudaMemsetAsync(C.b, 0, sizeof(T) * C.n, s), "coarse b = 0"))) return st;
    k_p_restrict_sf<T><<<(unsigned)std::min<int64_t>(L.op->n_cells, 152 * 16), 128, 0, s>>>(
        L.op->n_cells, L.op->d_map, C.op->d_map, (const T *)L.r, (const T *)L.inv_val, (T *)C.b, P);
  } else {
    k_h_restrict<T><<<grid1d(C.n), T256, 0, s>>>(hgrid(L, C), (const T *)L.r, (T *)C.b);
  }
  if ((st = cuda_status(cudaGetLastError(), "restrict"))) return st;
  if ((st = vcycle<T>(mg, l + 1, s))) return st;
  if (L.to_coarse == 1) {
    const PTransferParams P = ptransfer(L.op, C.op);
    if ((st = cuda_status(cudaMemsetAsync(L.t, 0, sizeof(T) * L.n, s), "t = 0"))) return st;
    k_p_prolongate_sf<T><<<(unsigned)std::min<int64_t>(L.op->n_cells, 152 * 16), 128, 0, s>>>(
        L.op->n_cells, L.op->d_map, C.op->d_map, (const T *)C.x, (T *)L.t, P);
    k_axpy<T><<<grid1d(L.n), T256, 0, s>>>(L.n, (T)1, (const T *)L.t, (T *)L.x);
  } else {
    k_h_prolongate_add<T><<<grid1d(L.n), T256, 0, s>>>(hgrid(L, C), (const T *)C.x,
                                                        (T *)L.x);
  }
  if ((st = cuda_status(cudaGetLastError(), "prolongate"))) return st;
  return chebyshev<T>(L, mg->degree, mg->range, false, prec, s);
}

// dst = M src (FP64 in and out): src -> level-0 b, V-cycle, level-0 x -> dst
mfgb_status mg_apply(mfgb_mg *mg, double *dst, const double *src, cudaStream_t s) {
  MgLevel &L = mg->levels[0];
  const unsigned g = grid1d(L.n);
  mfgb_status st;
  if (mg->precision == 32) {
    k_convert<float, double><<<g, T256, 0, s>>>(L.n, src, (float *)L.b);
    if ((st = vcycle<float>(mg, 0, s))) return st;
    k_convert<double, float><<<g, T256, 0, s>>>(L.n, (const float *)L.x, dst);
  } else {
    if ((st = cuda_status(cudaMemcpyAsync(L.b, src, sizeof(double) * L.n,
                                          cudaMemcpyDeviceToDevice, s),
                          "mg: b = src")))
      return st;
    if ((st = vcycle<double>(mg, 0, s))) return st;
    if ((st = cuda_status(cudaMemcpyAsync(dst, L.x, sizeof(double) * L.n,
                                          cudaMemcpyDeviceToDevice, s),
                          "mg: dst = x")))
      return st;
  }
  return cuda_status(cudaGetLastError(), "mg apply");
}

// lambda_max of Dinv A by power iteration (FP64 host-driven, set-up only)
mfgb_status estimate_lmax(MgLevel &L, int prec, int iters, double *lmax,
                          const double *dinv_given = nullptr) {
  const int64_t n = L.n;
  std::vector<double> h(n);
  uint64_t st64 = 0x9E3779B97F4A7C15ull;
  for (int64_t i = 0; i < n; ++i) {  // deterministic pseudo-random start
    st64 ^= st64 << 13; st64 ^= st64 >> 7; st64 ^= st64 << 17;
    h[i] = 0.5 + (double)(st64 >> 11) * (1.0 / 9007199254740992.0);
  }
  double *v = nullptr, *w = nullptr, *dinv = nullptr;
  mfgb_status st;
  if ((st = dalloc((void **)&v, sizeof(double) * n)) || (st = dalloc((void **)&w, sizeof(double) * n)) ||
      (st = dalloc((void **)&dinv, sizeof(double) * n))) {
    cudaFree(v); cudaFree(w); cudaFree(dinv);
    return st;
  }
  struct Free { double *a, *b, *c; ~Free() { cudaFree(a); cudaFree(b); cudaFree(c); } } fr{v, w, dinv};
  if ((st = cuda_status(cudaMemcpy(v, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice), "lmax init")))
    return st;
  if (L.op->n_constrained)
    k_set_constrained<double><<<grid1d(L.op->n_constrained), T256>>>(L.op->n_constrained,
                                                                      L.op->d_constrained, v, 0.0);
  if (dinv_given) {
    if ((st = cuda_status(cudaMemcpy(dinv, dinv_given, sizeof(double) * n, cudaMemcpyDeviceToDevice),
                          "lmax dinv")))
      return st;
  } else if ((st = mfgb_compute_diagonal(L.op, dinv, nullptr)) ||
             (st = cuda_status(invert_diagonal(n, dinv, nullptr), "invert diag"))) {
    return st;
  }
  double lam = 0;
  for (int it = 0; it < iters; ++it) {
    double nv = 0;
    if ((st = mfgb_dot(n, v, v, &nv, nullptr))) return st;
    const double inv = nv > 0 ? 1.0 / std::sqrt(nv) : 0.0;
    k_axpy<double><<<grid1d(n), T256>>>(n, inv - 1.0, v, v);  // v *= inv
    if (prec == 32) {  // the smoother's own FP32 operator, on a float copy
      k_convert<float, double><<<grid1d(n), T256>>>(n, v, (float *)L.t);
      if ((st = level_vmult(L.op, 32, L.d, L.t, nullptr))) return st;
      k_convert<double, float><<<grid1d(n), T256>>>(n, (const float *)L.d, w);
    } else if ((st = vmult_impl(L.op, w, v, MFGB_ARITH_FP64_DF, nullptr, nullptr, nullptr))) {
      return st;
    }
    if (L.op->n_constrained)  // power iteration on the unconstrained block
      k_set_constrained<double><<<grid1d(L.op->n_constrained), T256>>>(L.op->n_constrained,
                                                                        L.op->d_constrained, w, 0.0);
    k_scale_by<double><<<grid1d(n), T256>>>(n, dinv, w);
    double vw = 0;
    if ((st = mfgb_dot(n, v, w, &vw, nullptr))) return st;  // Rayleigh quotient (|v| = 1)
    lam = vw;
    std::swap(v, w);
  }
  fr.a = v; fr.b = w;
  *lmax = lam;
  return cuda_status(cudaGetLastError(), "lmax");
}

void free_mg(mfgb_mg *mg) {
  if (!mg) return;
  for (auto &L : mg->levels) {
    cudaFree(L.x); cudaFree(L.b); cudaFree(L.r); cudaFree(L.d); cudaFree(L.t);
    cudaFree(L.inv_diag); cudaFree(L.inv_val);
    if (L.op) mfgb_operator_destroy(L.op);
  }
  cudaFree(mg->coarse.A); cudaFree(mg->coarse.dinv); cudaFree(mg->coarse.work);
  cudaFree(mg->coarse.ids);
  cudaFree(mg->r); cudaFree(mg->z); cudaFree(mg->p); cudaFree(mg->v); cudaFree(mg->part);
  cudaFree(mg->scal);
  delete mg;
}

}  // namespace
}  // namespace mfgb

using namespace mfgb;

extern "C" mfgb_status mfgb_mg_setup(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                     mfgb_mg **out) {
  if (!fine || !prm || !out || (prm->precision != 32 && prm->precision != 64) ||
      prm->chebyshev_degree < 1 || prm->smoothing_range <= 1.0 || prm->eig_iterations < 1 ||
      prm->coarse_cells < 1) {
    set_error("mfgb_mg_setup: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *out = nullptr;
  mfgb_mg *mg = new mfgb_mg();
  mg->precision = prm->precision;
  mg->degree = prm->chebyshev_degree;
  mg->range = prm->smoothing_range;
  mg->coarse_tol = prm->coarse_tol > 0 ? prm->coarse_tol : 1e-12;
  // level boxes: p-coarsening by halving, then h-coarsening of Q1 by 2
  std::vector<mfgb_box_desc> boxes;
  std::vector<int> kinds, strides;
  mfgb_box_desc b = *fine;
  // every level keeps the fine level's geometry degree (coarse Q1 cells of a
  // deformed mesh would otherwise fold)
  b.geometry_degree = fine->geometry_degree > 0 ? fine->geometry_degree : fine->degree;
  boxes.push_back(b);
  strides.push_back(1);
  while (b.degree > 1) {
    b.degree = std::max(1, b.degree / 2);
    boxes.push_back(b);
    strides.push_back(1);
    kinds.push_back(1);
  }
  // h-levels: stride 2^l, ceil(n / 2^l) cells per axis (nested for any n)
  for (int s = 2; std::max({b.nx, b.ny, b.nz}) > prm->coarse_cells; s *= 2) {
    b.nx = (fine->nx + s - 1) / s;
    b.ny = (fine->ny + s - 1) / s;
    b.nz = (fine->nz + s - 1) / s;
    boxes.push_back(b);
    strides.push_back(s);
    kinds.push_back(2);
  }
  kinds.push_back(0);
  mfgb_status st = MFGB_OK;
  const size_t ts = tsize(prm->precision);
  for (size_t l = 0; l < boxes.size() && !st; ++l) {
    MgLevel L;
    L.box = boxes[l];
    L.to_coarse = kinds[l];
    L.bs = BoxStride{{fine->nx, fine->ny, fine->nz}, strides[l]};
    st = create_box_strided(&boxes[l], &L.bs, &L.op);
    if (st) break;
    L.n = L.op->n_dofs;
    mg->levels.push_back(L);
    MgLevel &M = mg->levels.back();
    if ((st = dalloc(&M.x, ts * M.n)) || (st = dalloc(&M.b, ts * M.n)) ||
        (st = dalloc(&M.r, ts * M.n)) || (st = dalloc(&M.d, ts * M.n)) ||
        (st = dalloc(&M.t, ts * M.n)) || (st = dalloc(&M.inv_diag, ts * M.n)))
      break;
    if (prm->precision == 32 && (st = ensure_g32(M.op))) break;
    if (prm->precision == 64 && (st = ensure_df(M.op))) break;
    // Jacobi in the V-cycle precision
    double *d64 = nullptr;
    if ((st = dalloc((void **)&d64, sizeof(double) * M.n))) break;
    st = mfgb_compute_diagonal(M.op, d64, nullptr);
    if (!st) st = cuda_status(invert_diagonal(M.n, d64, nullptr), "invert diag");
    if (!st) {
      if (prm->precision == 32)
        k_convert<float, double><<<grid1d(M.n), T256>>>(M.n, d64, (float *)M.inv_diag);
      else
        cudaMemcpy(M.inv_diag, d64, sizeof(double) * M.n, cudaMemcpyDeviceToDevice);
      st = cuda_status(cudaDeviceSynchronize(), "mg diag");
    }
    cudaFree(d64);
    if (st) break;
    if (M.to_coarse == 1) {  // 1/valence for the p-restriction
      if ((st = dalloc(&M.inv_val, ts * M.n))) break;
      cudaMemset(M.inv_val, 0, ts * M.n);
      const int64_t nm = M.op->n_cells * (int64_t)M.op->n * M.op->n * M.op->n;
      if (prm->precision == 32) {
        k_count_valence<float><<<grid1d(nm), T256>>>(nm, M.op->d_map, (float *)M.inv_val);
        k_invert_pos<float><<<grid1d(M.n), T256>>>(M.n, (float *)M.inv_val);
      } else {
        k_count_valence<double><<<grid1d(nm), T256>>>(nm, M.op->d_map, (double *)M.inv_val);
        k_invert_pos<double><<<grid1d(M.n), T256>>>(M.n, (double *)M.inv_val);
      }
      if ((st = cuda_status(cudaDeviceSynchronize(), "valence"))) break;
    }
    if (M.to_coarse != 0) {
      double lam = 0;
      if ((st = estimate_lmax(M, prm->precision, prm->eig_iterations, &lam))) break;
      M.lmax = 1.2 * lam;
    }
  }
  if (!st) {  // coarse matrix over the interior DoFs of the last level
    MgLevel &C = mg->levels.back();
    std::vector<uint8_t> cons(C.n, 0);
    std::vector<int64_t> hc(C.op->n_constrained);
    if (C.op->n_constrained)
      cudaMemcpy(hc.data(), C.op->d_constrained, sizeof(int64_t) * hc.size(), cudaMemcpyDeviceToHost);
    for (int64_t c : hc) cons[c] = 1;
    std::vector<int64_t> ids;
    for (int64_t i = 0; i < C.n; ++i)
      if (!cons[i]) ids.push_back(i);
    const int nc = (int)ids.size();
    if (nc > 4096) {
      set_error("mfgb_mg_setup: coarse problem too large for the one-CTA solver");
      st = MFGB_ERR_UNSUPPORTED;
    } else if (nc > 0) {
      std::vector<double> Ad((size_t)nc * nc), dinv(nc);
      double *e = nullptr, *y = nullptr;
      st = dalloc((void **)&e, sizeof(double) * C.n);
      if (!st) st = dalloc((void **)&y, sizeof(double) * C.n);
      std::vector<double> hy(C.n);
      for (int j = 0; j < nc && !st; ++j) {
        cudaMemset(e, 0, sizeof(double) * C.n);
        const double one = 1.0;
        cudaMemcpy(e + ids[j], &one, sizeof(double), cudaMemcpyHostToDevice);
        st = vmult_impl(C.op, y, e, MFGB_ARITH_FP64, nullptr, nullptr, nullptr);
        if (!st) st = cuda_status(cudaMemcpy(hy.data(), y, sizeof(double) * C.n, cudaMemcpyDeviceToHost), "coarse column");
        for (int i = 0; i < nc && !st; ++i) Ad[(size_t)i * nc + j] = hy[ids[i]];
      }
      cudaFree(e);
      cudaFree(y);
      for (int i = 0; i < nc; ++i) dinv[i] = Ad[(size_t)i * nc + i] > 0 ? 1.0 / Ad[(size_t)i * nc + i] : 1.0;
      if (!st && !(st = dalloc((void **)&mg->coarse.A, sizeof(double) * nc * nc)) &&
          !(st = dalloc((void **)&mg->coarse.dinv, sizeof(double) * nc)) &&
          !(st = dalloc((void **)&mg->coarse.work, sizeof(double) * 4 * nc)) &&
          !(st = dalloc((void **)&mg->coarse.ids, sizeof(int64_t) * nc))) {
        cudaMemcpy(mg->coarse.A, Ad.data(), sizeof(double) * nc * nc, cudaMemcpyHostToDevice);
        cudaMemcpy(mg->coarse.dinv, dinv.data(), sizeof(double) * nc, cudaMemcpyHostToDevice);
        cudaMemcpy(mg->coarse.ids, ids.data(), sizeof(int64_t) * nc, cudaMemcpyHostToDevice);
        mg->coarse.n = nc;
      }
    }
  }
  if (!st) st = cuda_status(cudaDeviceSynchronize(), "mg set-up");
  if (st) {
    free_mg(mg);
    return st;
  }
  *out = mg;
  return MFGB_OK;
}

// Learned smoother weights on the finest level: the Jacobi diagonal inside the
// Chebyshev smoother becomes D~ = sum_e w_e D_e (w_e > 0 per cell, e.g. the
// predicted lambda_max(D_e^-1 A_e)); d_cell_weights == NULL restores the plain
// diagonal.  lambda_max of D~^-1 A is re-estimated.
extern "C" mfgb_status mfgb_mg_set_smoother_weights(mfgb_mg *mg, const double *d_cell_weights) {
  if (!mg || mg->levels.empty()) {
    set_error("mfgb_mg_set_smoother_weights: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  MgLevel &L = mg->levels[0];
  if (L.to_coarse == 0) {
    set_error("mfgb_mg_set_smoother_weights: single-level hierarchy has no smoother");
    return MFGB_ERR_UNSUPPORTED;
  }
  double *d64 = nullptr;
  mfgb_status st = dalloc((void **)&d64, sizeof(double) * L.n);
  if (st) return st;
  if (d_cell_weights) {
    st = cuda_status(cudaMemset(d64, 0, sizeof(double) * L.n), "diag = 0");
    if (!st) st = cuda_status(weighted_diagonal(L.op, d_cell_weights, d64, nullptr), "weighted diag");
    if (!st)
      st = cuda_status(set_constrained(L.op->n_constrained, L.op->d_constrained, d64, 1.0, nullptr),
                       "weighted diag constrained");
  } else {
    st = mfgb_compute_diagonal(L.op, d64, nullptr);
  }
  if (!st) st = cuda_status(invert_diagonal(L.n, d64, nullptr), "invert diag");
  double lam = 0;
  if (!st) st = estimate_lmax(L, mg->precision, 20, &lam, d64);
  if (!st) {
    L.lmax = 1.2 * lam;
    if (mg->precision == 32)
      k_convert<float, double><<<grid1d(L.n), T256>>>(L.n, d64, (float *)L.inv_diag);
    else
      cudaMemcpy(L.inv_diag, d64, sizeof(double) * L.n, cudaMemcpyDeviceToDevice);
    st = cuda_status(cudaDeviceSynchronize(), "smoother weights");
  }
  cudaFree(d64);
  return st;
}

extern "C" mfgb_status mfgb_mg_destroy(mfgb_mg *mg) {
  free_mg(mg);
  return MFGB_OK;
}

extern "C" mfgb_status mfgb_mg_info(const mfgb_mg *mg, int *n_levels, int64_t *h_dofs,
                                    int *h_degree, double *h_lmax) {
  if (!mg) {
    set_error("mfgb_mg_info: null");
    return MFGB_ERR_INVALID_ARG;
  }
  if (n_levels) *n_levels = (int)mg->levels.size();
  for (size_t l = 0; l < mg->levels.size(); ++l) {
    if (h_dofs) h_dofs[l] = mg->levels[l].n;
    if (h_degree) h_degree[l] = mg->levels[l].box.degree;
    if (h_lmax) h_lmax[l] = mg->levels[l].lmax;
  }
  return MFGB_OK;
}

extern "C" mfgb_status mfgb_mg_vmult(mfgb_mg *mg, double *d_dst, const double *d_src,
                                     void *stream) {
  if (!mg || !d_dst || !d_src) {
    set_error("mfgb_mg_vmult: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  return mg_apply(mg, d_dst, d_src, (cudaStream_t)stream);
}

// FP64 PCG with the V-cycle as preconditioner (deal.II SolverCG semantics).
// One iteration = operator apply + update + V-cycle + dot + direction update,
// captured once into a CUDA graph and replayed; the host reads |r| after
// every iteration (a few microseconds against a V-cycle of milliseconds).
extern "C" mfgb_status mfgb_mg_cg_solve(const mfgb_operator *cop, mfgb_mg *mg, const double *d_b,
                                        double *d_x, const mfgb_cg_control *ctl,
                                        mfgb_solve_info *info, void *stream) {
  if (!cop || !mg || !d_b || !d_x || !ctl || !info || cop->n_dofs != mg->levels[0].n) {
    set_error("mfgb_mg_cg_solve: invalid argument (operator and hierarchy sizes must match)");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb_operator *op = const_cast<mfgb_operator *>(cop);
  const int64_t n = op->n_dofs;
  mfgb_status st;
  if (mg->outer_n != n) {
    cudaFree(mg->r); cudaFree(mg->z); cudaFree(mg->p); cudaFree(mg->v); cudaFree(mg->part);
    cudaFree(mg->scal);
    mg->r = mg->z = mg->p = mg->v = mg->part = mg->scal = nullptr;
    if ((st = dalloc((void **)&mg->r, sizeof(double) * n)) ||
        (st = dalloc((void **)&mg->z, sizeof(double) * n)) ||
        (st = dalloc((void **)&mg->p, sizeof(double) * n)) ||
        (st = dalloc((void **)&mg->v, sizeof(double) * n)) ||
        (st = dalloc((void **)&mg->part, sizeof(double) * (152 * 32 + 8))) ||
        (st = dalloc((void **)&mg->scal, sizeof(double) * 8)))
      return st;
    mg->outer_n = n;
  }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return cuda_status(cudaErrorUnknown, "stream create");
  struct SG { cudaStream_t s; ~SG() { cudaStreamDestroy(s); } } sg{s};
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, (cudaStream_t)stream);
  cudaStreamWaitEvent(s, ev, 0);
  cudaEventDestroy(ev);
  const int arith = ctl->arith;
  if (arith == MFGB_ARITH_FP64_DF && (st = ensure_df(op))) return st;
  const unsigned g = grid1d(n);
  double *r = mg->r, *z = mg->z, *p = mg->p, *v = mg->v, *part = mg->part, *scal = mg->scal;
  // scal: [0] r.z (current), [1] p.v, [2] r.z (new), [3] |r|^2
  auto dot_into = [&](const double *a, const double *b, int slot) {
    k_dot_partials<<<g, T256, 0, s>>>(n, a, b, part);
    k_sum_partials<<<1, T256, 0, s>>>(part, (int)g, scal + slot);
  };
  // r = b - A x ; z = M r ; p = z ; rz
  if ((st = vmult_impl(op, v, d_x, arith, nullptr, nullptr, s))) return st;
  k_residual<double><<<g, T256, 0, s>>>(n, d_b, v, r);
  dot_into(r, r, 3);
  double h[4];
  if ((st = cuda_status(cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, s), "pcg init")) ||
      (st = cuda_status(cudaStreamSynchronize(s), "pcg init")))
    return st;
  const double res0 = std::sqrt(h[3]);
  info->initial = info->last = res0;
  info->steps = 0;
  info->converged = 0;
  const double tol_eff = std::fmax(ctl->tol, ctl->reduce * res0);
  if (res0 <= tol_eff) { info->converged = 1; return MFGB_OK; }
  if (std::isnan(res0)) { set_error("mfgb_mg_cg_solve: NaN residual"); return MFGB_ERR_NONFINITE; }
  if ((st = mg_apply(mg, z, r, s))) return st;
  cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  dot_into(r, z, 0);

  // one iteration as a graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if ((st = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture")))
    return st;
  mfgb_status cap = vmult_impl(op, v, p, arith, nullptr, nullptr, s);
  if (!cap) {
    dot_into(p, v, 1);
    k_pcg_update<<<g, T256, 0, s>>>(n, d_x, r, p, v, scal, part);
    k_sum_partials<<<1, T256, 0, s>>>(part, (int)g, scal + 3);
    cap = mg_apply(mg, z, r, s);
  }
  if (!cap) {
    dot_into(r, z, 2);
    k_pcg_direction<<<g, T256, 0, s>>>(n, z, p, scal);
    k_copy_scalar<<<1, 32, 0, s>>>(scal, 2, 0);
  }
  const cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (cap) { if (graph) cudaGraphDestroy(graph); return cap; }
  if ((st = cuda_status(ce, "end capture"))) return st;
  if ((st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "instantiate"))) {
    cudaGraphDestroy(graph);
    return st;
  }
  mfgb_status result = MFGB_ERR_NOT_CONVERGED;
  for (int it = 1; it <= ctl->max_steps; ++it) {
    cudaError_t e = cudaGraphLaunch(exec, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, scal, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { result = cuda_status(e, "pcg iteration"); break; }
    const double res = std::sqrt(h[3]);
    info->steps = it;
    info->last = res;
    if (res <= tol_eff) { info->converged = 1; result = MFGB_OK; break; }
    if (std::isnan(res)) { set_error("mfgb_mg_cg_solve: NaN residual"); result = MFGB_ERR_NONFINITE; break; }
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  if (result == MFGB_OK || result == MFGB_ERR_NOT_CONVERGED) {
    const mfgb_status dev = mfgb_check_device_errors(s);
    if (dev) return dev;
  }
  if (result == MFGB_ERR_NOT_CONVERGED) set_error("mfgb_mg_cg_solve: max_steps reached");
  return result;
}

// FP32 operator on FP32 vectors (the multigrid levels' arithmetic)
extern "C" mfgb_status mfgb_vmult_f32(const mfgb_operator *cop, float *d_dst, const float *d_src,
                                      void *stream) {
  if (!cop || (cop->n_dofs > 0 && (!d_dst || !d_src)) || (const void *)d_dst == (const void *)d_src) {
    set_error("mfgb_vmult_f32: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb_operator *op = const_cast<mfgb_operator *>(cop);
  mfgb_status st = ensure_g32(op);
  if (st) return st;
  return level_vmult(op, 32, d_dst, d_src, (cudaStream_t)stream);
}
