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
#include "mfgb_mg_kernels.cuh"
#include "mfgb_mg_internal.h"

namespace mfgb {

namespace {

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

}  // namespace mfgb

namespace mfgb {

mfgb_status dalloc(void **p, size_t bytes) {
  *p = nullptr;
  if (!bytes) return MFGB_OK;
  if (alloc_hook_fails("multigrid allocation")) return MFGB_ERR_OUT_OF_MEMORY;
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

void mg_plan_levels(const mfgb_box_desc &fine, int coarse_cells, std::vector<mfgb_box_desc> &boxes,
                    std::vector<int> &kinds, std::vector<int> &strides) {
  boxes.clear();
  kinds.clear();
  strides.clear();
  mfgb_box_desc b = fine;
  // every level keeps the fine level's geometry degree (coarse Q1 cells of a
  // deformed mesh would otherwise fold)
  b.geometry_degree = fine.geometry_degree > 0 ? fine.geometry_degree : fine.degree;
  boxes.push_back(b);
  strides.push_back(1);
  while (b.degree > 1) {
    b.degree = std::max(1, b.degree / 2);
    boxes.push_back(b);
    strides.push_back(1);
    kinds.push_back(1);
  }
  // h-levels: stride 2^l, ceil(n / 2^l) cells per axis (nested for any n)
  for (int s = 2; std::max({b.nx, b.ny, b.nz}) > coarse_cells; s *= 2) {
    b.nx = (fine.nx + s - 1) / s;
    b.ny = (fine.ny + s - 1) / s;
    b.nz = (fine.nz + s - 1) / s;
    boxes.push_back(b);
    strides.push_back(s);
    kinds.push_back(2);
  }
  kinds.push_back(0);
}

namespace {

size_t tsize(int prec) { return prec == 32 ? sizeof(float) : sizeof(double); }

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
    p_transfer<T>(true, L.op->n_cells, L.op->d_map, C.op->d_map, (const T *)L.r,
                  (const T *)L.inv_val, (T *)C.b, P, s);
  } else {
    k_h_restrict<T><<<grid1d(C.n), T256, 0, s>>>(hgrid(L.box, L.bs, C.box), (const T *)L.r, (T *)C.b);
  }
  if ((st = cuda_status(cudaGetLastError(), "restrict"))) return st;
  if ((st = vcycle<T>(mg, l + 1, s))) return st;
  if (L.to_coarse == 1) {
    const PTransferParams P = ptransfer(L.op, C.op);
    if ((st = cuda_status(cudaMemsetAsync(L.t, 0, sizeof(T) * L.n, s), "t = 0"))) return st;
    p_transfer<T>(false, L.op->n_cells, L.op->d_map, C.op->d_map, (const T *)C.x, nullptr,
                  (T *)L.t, P, s);
    k_axpy<T><<<grid1d(L.n), T256, 0, s>>>(L.n, (T)1, (const T *)L.t, (T *)L.x);
  } else {
    k_h_prolongate_add<T><<<grid1d(L.n), T256, 0, s>>>(hgrid(L.box, L.bs, C.box), (const T *)C.x,
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

// v += (1/sqrt(*nv) - 1) v, i.e. v / |v| as the host formula 1/sqrt then axpy
// (0 for a zero vector)
__global__ void k_normalize(int64_t n, const double *__restrict__ nv, double *__restrict__ v) {
  const double s = *nv;
  const double a = (s > 0 ? 1.0 / sqrt(s) : 0.0) - 1.0;
  GRID_STRIDE(t, n) v[t] += a * v[t];
}

// lambda_max of Dinv A by power iteration (FP64, device scalars; set-up only)
mfgb_status estimate_lmax(MgLevel &L, int prec, int iters, double *lmax,
                          const double *dinv_given = nullptr) {
  const int64_t n = L.n;
  // scratch: dot partials, then |v|^2 and the Rayleigh quotient (device scalars:
  // the iteration runs without host synchronisation, one read at the end)
  const int np = dot_partials_count();
  double *v = nullptr, *w = nullptr, *dinv = nullptr, *scr = nullptr;
  mfgb_status st;
  if ((st = dalloc((void **)&v, sizeof(double) * n)) || (st = dalloc((void **)&w, sizeof(double) * n)) ||
      (st = dalloc((void **)&dinv, sizeof(double) * n)) ||
      (st = dalloc((void **)&scr, sizeof(double) * (np + 2)))) {
    cudaFree(v); cudaFree(w); cudaFree(dinv); cudaFree(scr);
    return st;
  }
  struct Free {
    double *a, *b, *c, *d;
    ~Free() { cudaFree(a); cudaFree(b); cudaFree(c); cudaFree(d); }
  } fr{v, w, dinv, scr};
  double *d_nv = scr + np, *d_vw = scr + np + 1;
  k_power_start<<<grid1d(n), T256>>>(n, v);  // deterministic pseudo-random start
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
  // the iterations on a stream of their own; after one plain iteration (which
  // also runs the kernels' one-time set-up), pairs of iterations (v -> w,
  // w -> v) are replayed from one CUDA graph: the set-up of a batch of
  // problems was bound by the launch latency of these small kernels
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    s = nullptr;
  }
  struct Stream {
    cudaStream_t s;
    ~Stream() { if (s) cudaStreamDestroy(s); }
  } sg{s};
  if ((st = cuda_status(cudaDeviceSynchronize(), "lmax set-up"))) return st;
  auto body = [&](double *vi, double *wo) -> mfgb_status {
    mfgb_status e;
    if ((e = cuda_status(dot_to_device(n, vi, vi, scr, d_nv, s), "lmax |v|"))) return e;
    k_normalize<<<grid1d(n), T256, 0, s>>>(n, d_nv, vi);  // v *= 1 / |v|
    if (prec == 32) {  // the smoother's own FP32 operator, on a float copy
      k_convert<float, double><<<grid1d(n), T256, 0, s>>>(n, vi, (float *)L.t);
      if ((e = level_vmult(L.op, 32, L.d, L.t, s))) return e;
      k_convert<double, float><<<grid1d(n), T256, 0, s>>>(n, (const float *)L.d, wo);
    } else if ((e = vmult_impl(L.op, wo, vi, MFGB_ARITH_FP64_DF, nullptr, nullptr, s))) {
      return e;
    }
    if (L.op->n_constrained)  // power iteration on the unconstrained block
      k_set_constrained<double><<<grid1d(L.op->n_constrained), T256, 0, s>>>(
          L.op->n_constrained, L.op->d_constrained, wo, 0.0);
    k_scale_by<double><<<grid1d(n), T256, 0, s>>>(n, dinv, wo);
    // Rayleigh quotient (|v| = 1)
    return cuda_status(dot_to_device(n, vi, wo, scr, d_vw, s), "lmax v.w");
  };
  int it = 0;
  if (iters > 0) {
    if ((st = body(v, w))) return st;
    std::swap(v, w);
    ++it;
  }
  if (s && iters - it >= 2) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      mfgb_status b = body(v, w);
      if (!b) b = body(w, v);
      const cudaError_t ec = cudaStreamEndCapture(s, &g);
      if (!b && ec == cudaSuccess && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
        for (; it + 2 <= iters; it += 2)
          if ((st = cuda_status(cudaGraphLaunch(ge, s), "lmax graph"))) break;
        if (!st) st = cuda_status(cudaStreamSynchronize(s), "lmax graph");
      }
      if (ge) cudaGraphExecDestroy(ge);
      if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();  // a capture that did not work leaves the plain loop below
    if (st) return st;
  }
  for (; it < iters; ++it) {
    if ((st = body(v, w))) return st;
    std::swap(v, w);
  }
  if ((st = cuda_status(s ? cudaStreamSynchronize(s) : cudaDeviceSynchronize(), "lmax"))) return st;
  fr.a = v; fr.b = w;
  if (iters > 0 &&
      (st = cuda_status(cudaMemcpy(&lam, d_vw, sizeof(double), cudaMemcpyDeviceToHost), "lmax")))
    return st;
  *lmax = lam;
  return cuda_status(cudaGetLastError(), "lmax");
}

void free_mg(mfgb_mg *mg) {
  if (!mg) return;
  for (auto &L : mg->levels) {
    cudaFree(L.x); cudaFree(L.b); cudaFree(L.r); cudaFree(L.d); cudaFree(L.t);
    cudaFree(L.inv_diag); cudaFree(L.inv_val);
    if (L.op && !L.borrowed) mfgb_operator_destroy(L.op);
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

static mfgb_status mg_setup_impl(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                 mfgb_mg **out, mfgb_operator *fine_op, bool lmax = true);

extern "C" mfgb_status mfgb_mg_setup(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                     mfgb_mg **out) {
  return mg_setup_impl(fine, prm, out, nullptr);
}

// The finest level borrows the caller's operator (its geometric factors are
// not computed a second time); the operator must outlive the hierarchy.
namespace mfgb {
// the hierarchy without the lambda_max estimates (levels[l].lmax = 0): the
// batched set-up estimates them for all problems at once
mfgb_status mg_setup_without_lmax(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                  mfgb_mg **out) {
  return mg_setup_impl(fine, prm, out, nullptr, false);
}
}  // namespace mfgb

extern "C" mfgb_status mfgb_mg_setup_shared(const mfgb_operator *fine_op,
                                            const mfgb_mg_params *prm, mfgb_mg **out) {
  if (!fine_op || !fine_op->is_box || fine_op->quadrature != 0 ||
      fine_op->n_dofs != ((int64_t)fine_op->degree * fine_op->box.nx + 1) *
                             ((int64_t)fine_op->degree * fine_op->box.ny + 1) *
                             ((int64_t)fine_op->degree * fine_op->box.nz + 1)) {
    set_error("mfgb_mg_setup_shared: needs a GLL-collocated box operator");
    return MFGB_ERR_INVALID_ARG;
  }
  return mg_setup_impl(&fine_op->box, prm, out, const_cast<mfgb_operator *>(fine_op));
}

static mfgb_status mg_setup_impl(const mfgb_box_desc *fine, const mfgb_mg_params *prm,
                                 mfgb_mg **out, mfgb_operator *fine_op, bool lmax) {
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
  mg_plan_levels(*fine, prm->coarse_cells, boxes, kinds, strides);
  mfgb_status st = MFGB_OK;
  const size_t ts = tsize(prm->precision);
  for (size_t l = 0; l < boxes.size() && !st; ++l) {
    MgLevel L;
    L.box = boxes[l];
    L.to_coarse = kinds[l];
    L.bs = BoxStride{{fine->nx, fine->ny, fine->nz}, strides[l]};
    if (l == 0 && fine_op && (fine_op->box.geometry_degree == 0 ||
                              fine_op->box.geometry_degree == boxes[0].geometry_degree)) {
      L.op = fine_op;  // the same box, degree and geometry interpolant
      L.borrowed = true;
    } else {
      st = create_box_strided(&boxes[l], &L.bs, &L.op);
    }
    if (st) break;
    L.n = L.op->n_dofs;
    mg->levels.push_back(L);
    MgLevel &M = mg->levels.back();
    if ((st = dalloc(&M.x, ts * M.n)) || (st = dalloc(&M.b, ts * M.n)) ||
        (st = dalloc(&M.r, ts * M.n)) || (st = dalloc(&M.d, ts * M.n)) ||
        (st = dalloc(&M.t, ts * M.n)) || (st = dalloc(&M.inv_diag, ts * M.n)))
      break;
    if (prm->precision == 32 && (st = ensure_g32(M.op))) break;
    if (prm->precision == 64 && (st = ensure_arith(M.op, MFGB_ARITH_FP64_DF))) break;
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
    if (M.to_coarse != 0 && lmax) {
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
      // columns A e_j in blocks of up to 32 MB of unit vectors: the applies are
      // queued without host synchronisation, one copy back per block
      const int64_t cb = std::max<int64_t>(1, std::min<int64_t>(nc, (4 << 20) / C.n));
      double *e = nullptr, *y = nullptr;
      st = dalloc((void **)&e, sizeof(double) * C.n * cb);
      if (!st) st = dalloc((void **)&y, sizeof(double) * C.n * cb);
      std::vector<double> hy((size_t)C.n * cb), he((size_t)C.n * cb);
      for (int j0 = 0; j0 < nc && !st; j0 += (int)cb) {
        const int nb = (int)std::min<int64_t>(cb, nc - j0);
        std::fill(he.begin(), he.begin() + (size_t)nb * C.n, 0.0);
        for (int jj = 0; jj < nb; ++jj) he[(size_t)jj * C.n + ids[j0 + jj]] = 1.0;
        st = cuda_status(cudaMemcpy(e, he.data(), sizeof(double) * C.n * nb, cudaMemcpyHostToDevice),
                         "coarse unit vectors");
        for (int jj = 0; jj < nb && !st; ++jj)
          st = vmult_impl(C.op, y + (size_t)jj * C.n, e + (size_t)jj * C.n, MFGB_ARITH_FP64, nullptr,
                          nullptr, nullptr);
        if (!st)
          st = cuda_status(cudaMemcpy(hy.data(), y, sizeof(double) * C.n * nb, cudaMemcpyDeviceToHost),
                           "coarse columns");
        for (int jj = 0; jj < nb && !st; ++jj)
          for (int i = 0; i < nc; ++i) Ad[(size_t)i * nc + j0 + jj] = hy[(size_t)jj * C.n + ids[i]];
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
  if ((st = ensure_arith(op, arith))) return st;
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
