// mfgb_batch.cu -- many independent BP5 problems (each with its own box mesh,
// degree, deformation and right-hand side) solved together: FP64 CG with
// per-problem scalars, preconditioned by a batched FP32 p-/h-multigrid
// V-cycle (the single-problem method of mfgb_mg.cu, problem by problem).
//
// GB300 layout:
//   * depth vectors: the problems' level-l vectors are concatenated (problem
//     order) into one vector per depth l;
//   * union operators: on each depth, the cells of all problems of one degree
//     form one operator whose map points into the depth vector, so a single
//     BK5 launch per degree applies every problem's operator (small problems
//     share launches with large ones instead of each paying launch latency);
//   * chunk tables: element-wise kernels run one CTA per chunk of <= 4096
//     entries lying inside one problem, so each CTA reads that problem's
//     Chebyshev coefficients or CG scalars; dot products are per-chunk
//     partials summed per problem in a fixed order (deterministic);
//   * coarse solves: every problem's coarsest level is a small Q1 system whose
//     FP64 inverse is formed at set-up; all of them run in one launch at the
//     bottom of the V-cycle (a problem's coarse solve only has to follow its
//     restriction and precede its prolongation, whatever its depth);
//   * one CG iteration of the whole batch is one CUDA graph, replayed until
//     every problem has converged or failed; converged problems keep their
//     iterate (their updates are skipped).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"
#include "mfgb_mg_kernels.cuh"
#include "mfgb_mg_internal.h"

namespace mfgb {
namespace {

constexpr int CHUNK = 4096;

struct Chunk {
  int64_t start;  // first entry (index into the depth vector)
  int32_t len;
  int32_t part;   // index of the owning part (or h-transfer entry)
};

struct HPart {
  HGrid g;
  int64_t off_f, off_c;  // node 0 of the fine / coarse part in its depth vector
};

struct CoarseDesc {
  const float *b;
  float *x;
  const double *Ainv;  // [nc][nc]
  const int32_t *ids;  // interior DoFs (local indices)
  int nc;
  int n;               // DoFs of the part (x is zeroed over all of them)
};

struct BScal {
  double rz, rz_new, pap, res0, res, tol_eff;
  int its, done;  // done: 0 running, 1 converged, 2 failed (max_steps or NaN)
};

#define CHUNK_LOOP(c, t)                                                             \
  const Chunk c = ch[blockIdx.x];                                                    \
  for (int64_t t = c.start + threadIdx.x, t##_end = c.start + c.len; t < t##_end; \
       t += blockDim.x)

__global__ void kb_map_offset(int64_t n, const uint32_t *__restrict__ src, uint32_t *__restrict__ dst,
                              uint32_t off) {
  GRID_STRIDE(t, n) {
    const uint32_t v = src[t];
    dst[t] = v == MFGB_INVALID_DOF ? MFGB_INVALID_DOF : v + off;
  }
}

__global__ void kb_offset_i64(int64_t n, const int64_t *__restrict__ src, int64_t *__restrict__ dst,
                              int64_t off) {
  GRID_STRIDE(t, n) dst[t] = src[t] + off;
}

// ---- batched Chebyshev (FP32), coefficients per part: [1/theta, c1_1, c2_1, ...]
__global__ void __launch_bounds__(T256)
    kb_cheb_first_zero(const Chunk *__restrict__ ch, const float *__restrict__ b,
                       const float *__restrict__ dinv, float *__restrict__ x, float *__restrict__ d,
                       float *__restrict__ r, const float *__restrict__ coef, int cs) {
  const float it = coef[(int64_t)ch[blockIdx.x].part * cs];
  CHUNK_LOOP(c, t) {
    const float bt = b[t];
    const float dt = it * dinv[t] * bt;
    r[t] = bt;
    d[t] = dt;
    x[t] = dt;
  }
}

__global__ void __launch_bounds__(T256)
    kb_cheb_first(const Chunk *__restrict__ ch, const float *__restrict__ b,
                  const float *__restrict__ ax, const float *__restrict__ dinv, float *__restrict__ x,
                  float *__restrict__ d, float *__restrict__ r, const float *__restrict__ coef,
                  int cs) {
  const float it = coef[(int64_t)ch[blockIdx.x].part * cs];
  CHUNK_LOOP(c, t) {
    const float rt = b[t] - ax[t];
    const float dt = it * dinv[t] * rt;
    r[t] = rt;
    d[t] = dt;
    x[t] += dt;
  }
}

__global__ void __launch_bounds__(T256)
    kb_cheb_step(const Chunk *__restrict__ ch, const float *__restrict__ ad,
                 const float *__restrict__ dinv, float *__restrict__ x, float *__restrict__ d,
                 float *__restrict__ r, const float *__restrict__ coef, int cs, int j) {
  const float *cf = coef + (int64_t)ch[blockIdx.x].part * cs;
  const float c1 = cf[2 * j - 1], c2 = cf[2 * j];
  CHUNK_LOOP(c, t) {
    const float rt = r[t] - ad[t];
    const float dt = c1 * d[t] + c2 * dinv[t] * rt;
    r[t] = rt;
    d[t] = dt;
    x[t] += dt;
  }
}

__global__ void __launch_bounds__(T256)
    kb_residual(const Chunk *__restrict__ ch, const float *__restrict__ b,
                const float *__restrict__ ax, float *__restrict__ r) {
  CHUNK_LOOP(c, t) r[t] = b[t] - ax[t];
}

__global__ void __launch_bounds__(T256)
    kb_add(const Chunk *__restrict__ ch, const float *__restrict__ t_, float *__restrict__ x) {
  CHUNK_LOOP(c, t) x[t] += t_[t];
}

__global__ void __launch_bounds__(T256)
    kb_h_prolongate_add(const Chunk *__restrict__ ch, const HPart *__restrict__ hp,
                        const float *__restrict__ xc, float *__restrict__ xf) {
  const HPart h = hp[ch[blockIdx.x].part];
  CHUNK_LOOP(c, t) h_prolongate_node(h.g, t - h.off_f, xc + h.off_c, xf + h.off_f);
}

__global__ void __launch_bounds__(T256)
    kb_h_restrict(const Chunk *__restrict__ ch, const HPart *__restrict__ hp,
                  const float *__restrict__ rf, float *__restrict__ rc) {
  const HPart h = hp[ch[blockIdx.x].part];
  CHUNK_LOOP(c, t) h_restrict_node(h.g, t - h.off_c, rf + h.off_f, rc + h.off_c);
}

// x = A^-1 b on the interior DoFs of one coarsest part per CTA (FP64)
__global__ void __launch_bounds__(T256) kb_coarse(const CoarseDesc *__restrict__ cd) {
  extern __shared__ double sb[];
  const CoarseDesc c = cd[blockIdx.x];
  for (int i = threadIdx.x; i < c.n; i += blockDim.x) c.x[i] = 0.f;
  for (int i = threadIdx.x; i < c.nc; i += blockDim.x) sb[i] = (double)c.b[c.ids[i]];
  __syncthreads();
  for (int i = threadIdx.x; i < c.nc; i += blockDim.x) {
    const double *row = c.Ainv + (int64_t)i * c.nc;
    double s = 0.0;
    for (int j = 0; j < c.nc; ++j) s = fma(row[j], sb[j], s);
    c.x[c.ids[i]] = (float)s;
  }
}

// ---- outer FP64 CG with per-problem scalars -------------------------------
__device__ __forceinline__ double cta_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < T256 / 32; ++w) s += sh[w];
  return s;  // valid in thread 0
}

__global__ void __launch_bounds__(T256)
    kb_dot(const Chunk *__restrict__ ch, const double *__restrict__ a, const double *__restrict__ b,
           double *__restrict__ part) {
  __shared__ double sh[T256 / 32];
  double s = 0;
  CHUNK_LOOP(c, t) s = fma(a[t], b[t], s);
  s = cta_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// ---- power iterations for lambda_max(Dinv A) of every part of a depth -------
// (the single-problem estimate of mfgb_mg.cu on all parts at once; per-part
// sums accumulate by atomics into acc[part])
__global__ void __launch_bounds__(T256)
    kb_pi_start(const Chunk *__restrict__ ch, const int64_t *__restrict__ poff, double *__restrict__ v) {
  CHUNK_LOOP(c, t) v[t] = power_start_value((uint64_t)(t - poff[c.part]));
}

__global__ void __launch_bounds__(T256)
    kb_pi_dot(const Chunk *__restrict__ ch, const double *__restrict__ a,
              const double *__restrict__ b, double *__restrict__ acc) {
  __shared__ double sh[T256 / 32];
  double s = 0;
  CHUNK_LOOP(c, t) s = fma(a[t], b[t], s);
  s = cta_sum(s, sh);
  if (threadIdx.x == 0) atomicAdd(acc + ch[blockIdx.x].part, s);
}

// v /= |v| per part (the single-problem normalisation), and its float copy
__global__ void __launch_bounds__(T256)
    kb_pi_normalize(const Chunk *__restrict__ ch, const double *__restrict__ nv,
                    double *__restrict__ v, float *__restrict__ vf) {
  const double q = nv[ch[blockIdx.x].part];
  const double a = (q > 0 ? 1.0 / sqrt(q) : 0.0) - 1.0;
  CHUNK_LOOP(c, t) {
    v[t] += a * v[t];
    vf[t] = (float)v[t];
  }
}

// w = Dinv (A v) from the FP32 apply
__global__ void __launch_bounds__(T256)
    kb_pi_post(const Chunk *__restrict__ ch, const float *__restrict__ av,
               const float *__restrict__ inv_diag, double *__restrict__ w) {
  CHUNK_LOOP(c, t) w[t] = (double)av[t] * (double)inv_diag[t];
}

// CTA b handles problem pid[b]: the sum of its chunk partials cbeg[b] .. cbeg[b+1]
__device__ __forceinline__ double problem_sum(const int *__restrict__ cbeg,
                                              const double *__restrict__ part, double *sh) {
  const int b = blockIdx.x;
  double s = 0;
  for (int i = cbeg[b] + threadIdx.x; i < cbeg[b + 1]; i += blockDim.x) s += part[i];
  return cta_sum(s, sh);
}

__global__ void __launch_bounds__(T256)
    kb_sum_pap(const int *__restrict__ cbeg, const int *__restrict__ pid,
               const double *__restrict__ part, BScal *__restrict__ sc) {
  __shared__ double sh[T256 / 32];
  const double s = problem_sum(cbeg, part, sh);
  if (threadIdx.x == 0) sc[pid[blockIdx.x]].pap = s;
}

__global__ void __launch_bounds__(T256)
    kb_sum_rz(const int *__restrict__ cbeg, const int *__restrict__ pid,
              const double *__restrict__ part, BScal *__restrict__ sc) {
  __shared__ double sh[T256 / 32];
  const double s = problem_sum(cbeg, part, sh);
  if (threadIdx.x == 0) sc[pid[blockIdx.x]].rz_new = s;
}

// initial residual norms: tol_eff = max(tol, reduce |r0|)
__global__ void __launch_bounds__(T256)
    kb_init(const int *__restrict__ cbeg, const int *__restrict__ pid,
            const double *__restrict__ part, BScal *__restrict__ sc, double tol, double reduce) {
  __shared__ double sh[T256 / 32];
  const double rr = problem_sum(cbeg, part, sh);
  if (threadIdx.x == 0) {
    BScal &q = sc[pid[blockIdx.x]];
    const double res = sqrt(rr);
    q.res0 = q.res = res;
    q.tol_eff = fmax(tol, reduce * res);
    q.its = 0;
    q.done = isnan(res) ? 2 : (res <= q.tol_eff ? 1 : 0);
  }
}

__global__ void kb_init_rz(int n, BScal *__restrict__ sc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) sc[p].rz = sc[p].rz_new;
}

// x += alpha p; r -= alpha v (alpha = rz / pAp); per-chunk |r|^2
__global__ void __launch_bounds__(T256)
    kb_update(const Chunk *__restrict__ ch, double *__restrict__ x, double *__restrict__ r,
              const double *__restrict__ p, const double *__restrict__ v,
              const BScal *__restrict__ sc, double *__restrict__ part) {
  __shared__ double sh[T256 / 32];
  const BScal &q = sc[ch[blockIdx.x].part];
  double s = 0;
  if (!q.done) {
    const double alpha = q.rz / q.pap;
    CHUNK_LOOP(c, t) {
      x[t] = fma(alpha, p[t], x[t]);
      const double rt = fma(-alpha, v[t], r[t]);
      r[t] = rt;
      s = fma(rt, rt, s);
    }
  }
  s = cta_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// |r| test per problem (deal.II SolverCG / ReductionControl): converged when
// |r| <= tol_eff, failed at max_steps or NaN; counts the problems still running
__global__ void __launch_bounds__(T256)
    kb_sum_check(const int *__restrict__ cbeg, const int *__restrict__ pid,
                 const double *__restrict__ part, BScal *__restrict__ sc, int max_steps,
                 int *__restrict__ active, const int64_t *__restrict__ pdofs,
                 unsigned long long *__restrict__ active_dofs) {
  __shared__ double sh[T256 / 32];
  const double rr = problem_sum(cbeg, part, sh);
  if (threadIdx.x == 0) {
    const int p = pid[blockIdx.x];
    BScal &q = sc[p];
    if (!q.done) {
      const double res = sqrt(rr);
      q.res = res;
      q.its += 1;
      if (res <= q.tol_eff) {
        q.done = 1;
      } else if (q.its >= max_steps || isnan(res)) {
        q.done = 2;
      } else {
        atomicAdd(active, 1);
        atomicAdd(active_dofs, (unsigned long long)pdofs[p]);
      }
    }
  }
}

__global__ void kb_zero_active(int *active, unsigned long long *active_dofs) {
  *active = 0;
  *active_dofs = 0ull;
}

// the while-loop condition of a launch plan's graph: go on while problems run,
// they still hold more than `threshold` DoFs (else the host gathers a smaller
// plan), and the launch has run fewer than max_iter iterations (a hard bound)
__global__ void kb_continue(cudaGraphConditionalHandle h, const int *active,
                            const unsigned long long *active_dofs, unsigned long long threshold,
                            int *iter, int max_iter) {
  const int it = *iter + 1;
  *iter = it;
  cudaGraphSetConditional(h, (*active > 0 && *active_dofs > threshold && it < max_iter) ? 1u : 0u);
}

// p = z + beta p (beta = rz_new / rz) for running problems
__global__ void __launch_bounds__(T256)
    kb_direction(const Chunk *__restrict__ ch, const double *__restrict__ z, double *__restrict__ p,
                 const BScal *__restrict__ sc) {
  const BScal &q = sc[ch[blockIdx.x].part];
  if (q.done) return;
  const double beta = q.rz_new / q.rz;
  CHUNK_LOOP(c, t) p[t] = fma(beta, p[t], z[t]);
}

__global__ void kb_roll(int n, BScal *__restrict__ sc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n && !sc[p].done) sc[p].rz = sc[p].rz_new;
}

__global__ void __launch_bounds__(T256)
    kb_residual64(const Chunk *__restrict__ ch, const double *__restrict__ b,
                  const double *__restrict__ v, double *__restrict__ r) {
  CHUNK_LOOP(c, t) r[t] = b[t] - v[t];
}

__global__ void __launch_bounds__(T256)
    kb_copy64(const Chunk *__restrict__ ch, const double *__restrict__ a, double *__restrict__ b) {
  CHUNK_LOOP(c, t) b[t] = a[t];
}

// ---- host-side structures -------------------------------------------------
struct Part {
  int problem = 0;
  int64_t off = 0, n = 0, n_cells = 0, n_constrained = 0;
  int degree = 1;
  int kind = 0;          // 1 p-transfer to the next depth, 2 h-transfer, 0 coarsest
  mfgb_box_desc box{};
  BoxStride bs{};
  int group = -1;        // union operator on this depth, -1 none
  int64_t cell_off = 0;  // first cell in the union operator
  int64_t cons_off = 0;  // first entry in the depth's constrained list
  double lmax = 0;
};

struct PGroup {
  int g = 0;                   // union operator of the fine degree (its map is map_f)
  uint32_t *map_c = nullptr;   // coarse maps of the same cells, depth+1 offsets
  PTransferParams P{};
};

// What one batched CG iteration launches on one depth, for a set of problems:
// the union operators, identity rows, chunk tables and transfer tables.
struct DepthPlan {
  std::vector<mfgb_operator *> groups;
  const int64_t *d_cons = nullptr;
  int64_t n_cons = 0;
  const Chunk *d_cheb = nullptr, *d_pch = nullptr, *d_hfine = nullptr, *d_hcoarse = nullptr;
  int n_cheb = 0, n_pch = 0, n_hfine = 0, n_hcoarse = 0;
  std::vector<PGroup> pgroups;
  const HPart *d_hp = nullptr;
};

// A plan: every problem (built at set-up), or the problems still running
// (gathered from the full plan's arrays while solving: the depth vectors and the
// maps' offsets into them stay as they are).
struct Plan {
  std::vector<DepthPlan> depth;
  const CoarseDesc *d_coarse = nullptr;
  int n_coarse = 0, coarse_smem = 0;
  const Chunk *d_all = nullptr;  // outer CG chunks (depth 0)
  int n_all = 0;
  const int *d_cbeg = nullptr, *d_pid = nullptr;
  int n_prob = 0;
  int64_t dofs = 0;              // depth-0 DoFs of its problems
  bool owns = false;             // a gathered plan owns what it points to
  std::vector<void *> mem;
};

struct Depth {
  int64_t n = 0;
  std::vector<Part> parts;
  std::vector<mfgb_operator *> groups;
  int64_t *d_cons = nullptr;
  int64_t n_cons = 0;
  float *x = nullptr, *b = nullptr, *r = nullptr, *d = nullptr, *t = nullptr, *inv_diag = nullptr,
        *inv_val = nullptr;
  Chunk *d_cheb = nullptr;   // non-coarsest parts
  int n_cheb = 0;
  Chunk *d_pch = nullptr;    // parts with a p-transfer to depth+1
  int n_pch = 0;
  float *d_coef = nullptr;   // [parts][cs]
  std::vector<PGroup> pgroups;
  HPart *d_hp = nullptr;
  Chunk *d_hfine = nullptr;  // fine nodes of h-transfer parts (this depth)
  int n_hfine = 0;
  Chunk *d_hcoarse = nullptr;  // their coarse nodes (depth+1)
  int n_hcoarse = 0;
};

int64_t box_dofs(const mfgb_box_desc &b) {
  return ((int64_t)b.degree * b.nx + 1) * ((int64_t)b.degree * b.ny + 1) *
         ((int64_t)b.degree * b.nz + 1);
}

int64_t box_boundary(const mfgb_box_desc &b) {
  const int64_t X = (int64_t)b.degree * b.nx + 1, Y = (int64_t)b.degree * b.ny + 1,
                Z = (int64_t)b.degree * b.nz + 1;
  const int64_t ix = std::max<int64_t>(0, X - 2), iy = std::max<int64_t>(0, Y - 2),
                iz = std::max<int64_t>(0, Z - 2);
  return X * Y * Z - ix * iy * iz;
}

void append_chunks(std::vector<Chunk> &v, int64_t start, int64_t n, int part) {
  for (int64_t s = 0; s < n; s += CHUNK)
    v.push_back(Chunk{start + s, (int32_t)std::min<int64_t>(CHUNK, n - s), part});
}

template <class T>
mfgb_status upload(T **d, const std::vector<T> &h) {
  *d = nullptr;
  if (h.empty()) return MFGB_OK;
  mfgb_status st = dalloc((void **)d, sizeof(T) * h.size());
  if (st) return st;
  return cuda_status(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice),
                     "batch upload");
}

// inverse of an SPD matrix (Cholesky, FP64); false if not positive definite
bool spd_inverse(int n, const std::vector<double> &A, std::vector<double> &inv) {
  std::vector<double> L(A);
  for (int j = 0; j < n; ++j) {
    double d = L[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= L[(size_t)j * n + k] * L[(size_t)j * n + k];
    if (!(d > 0)) return false;
    d = std::sqrt(d);
    L[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = L[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
      L[(size_t)i * n + j] = s / d;
    }
  }
  inv.assign((size_t)n * n, 0.0);
  std::vector<double> y(n);
  for (int c = 0; c < n; ++c) {  // solve L L^T x = e_c
    for (int i = 0; i < n; ++i) {
      double s = i == c ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) s -= L[(size_t)i * n + k] * y[k];
      y[i] = s / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * inv[(size_t)k * n + c];
      inv[(size_t)i * n + c] = s / L[(size_t)i * n + i];
    }
  }
  return true;
}

}  // namespace
}  // namespace mfgb

struct mfgb_batch {
  int n_problems = 0;
  int cheb_degree = 5;
  int cs = 0;  // coefficients per part
  std::vector<mfgb_box_desc> boxes;
  std::vector<mfgb::Depth> depth;
  // coarse solves
  mfgb::CoarseDesc *d_coarse = nullptr;
  int n_coarse = 0;
  int coarse_smem = 0;
  double *d_Ainv = nullptr;
  int32_t *d_cids = nullptr;
  std::vector<mfgb::CoarseDesc> coarse_host;  // per problem, for gathered plans
  // outer CG (depth 0, every problem)
  mfgb::Chunk *d_all = nullptr;
  int n_all = 0;
  int *d_cbeg = nullptr, *d_pid = nullptr;
  mfgb::Plan full;
  double *r = nullptr, *z = nullptr, *p = nullptr, *v = nullptr, *part = nullptr;
  mfgb::BScal *d_scal = nullptr;
  int *d_active = nullptr;
  int *h_active = nullptr;  // pinned
  // device-side loop of the solve: DoFs of each problem, DoFs of the running
  // problems, iterations of the current graph launch
  int64_t *d_pdofs = nullptr;
  unsigned long long *d_active_dofs = nullptr;
  int *d_iter = nullptr;
  int last_launches = 0;  // graph launches of the last solve
  int last_replans = 0;     // plans gathered during the last solve
};

namespace mfgb {
namespace {

void free_batch(mfgb_batch *B) {
  if (!B) return;
  for (auto &D : B->depth) {
    for (auto *op : D.groups) mfgb_operator_destroy(op);
    for (auto &pg : D.pgroups) cudaFree(pg.map_c);
    cudaFree(D.d_cons); cudaFree(D.x); cudaFree(D.b); cudaFree(D.r); cudaFree(D.d); cudaFree(D.t);
    cudaFree(D.inv_diag); cudaFree(D.inv_val); cudaFree(D.d_cheb); cudaFree(D.d_pch);
    cudaFree(D.d_coef); cudaFree(D.d_hp); cudaFree(D.d_hfine); cudaFree(D.d_hcoarse);
  }
  cudaFree(B->d_coarse); cudaFree(B->d_Ainv); cudaFree(B->d_cids);
  cudaFree(B->d_all); cudaFree(B->d_cbeg); cudaFree(B->d_pid);
  cudaFree(B->r); cudaFree(B->z); cudaFree(B->p); cudaFree(B->v); cudaFree(B->part);
  cudaFree(B->d_scal); cudaFree(B->d_active);
  cudaFree(B->d_pdofs); cudaFree(B->d_active_dofs); cudaFree(B->d_iter);
  if (B->h_active) cudaFreeHost(B->h_active);
  delete B;
}

mfgb_operator *union_shell(int degree, int64_t n_dofs) {
  mfgb_operator *op = new mfgb_operator();
  op->degree = degree;
  op->n = degree + 1;
  gll_nodes(op->n, op->gll_x, op->gll_w);
  derivative_matrix(op->n, op->gll_x, op->D);
  op->n_dofs = n_dofs;
  return op;
}

void free_plan(Plan &P) {
  if (!P.owns) return;
  for (auto &D : P.depth) {
    for (auto *op : D.groups) mfgb_operator_destroy(op);
    for (auto &pg : D.pgroups) cudaFree(pg.map_c);
  }
  for (void *m : P.mem) cudaFree(m);
  P = Plan();
}

// dst = A src on one depth (FP32, union operators + identity rows)
mfgb_status apply32(const Depth &V, const DepthPlan &D, const float *src, float *dst,
                    cudaStream_t s) {
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(dst, 0, sizeof(float) * V.n, s), "batch A32: dst = 0")))
    return st;
  for (const mfgb_operator *op : D.groups)
    if ((st = cuda_status(bk5_f32(op->n, op->n_cells, op->d_map, op->d_G32, src, dst, op->D,
                                  nullptr, nullptr, s),
                          "batch A32 kernel")))
      return st;
  if (D.n_cons)
    k_copy_constrained<float><<<grid1d(D.n_cons), T256, 0, s>>>(D.n_cons, D.d_cons, src, dst);
  return cuda_status(cudaGetLastError(), "batch A32 constrained");
}

// dst = A src on depth 0 in FP64 (double-float union operators)
mfgb_status apply64(const mfgb_batch *B, const Plan &P, const double *src, double *dst,
                    cudaStream_t s) {
  const DepthPlan &D = P.depth[0];
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(dst, 0, sizeof(double) * B->depth[0].n, s),
                        "batch A: dst = 0")))
    return st;
  for (mfgb_operator *op : D.groups)
    if ((st = apply_add_impl(op, dst, src, MFGB_ARITH_FP64_DF, s, nullptr))) return st;
  return cuda_status(copy_constrained(D.n_cons, D.d_cons, src, dst, s), "batch A constrained");
}

mfgb_status chebyshev_b(const mfgb_batch *B, const Depth &V, const DepthPlan &D, bool zero_start,
                        cudaStream_t s) {
  mfgb_status st;
  if (zero_start) {
    kb_cheb_first_zero<<<D.n_cheb, T256, 0, s>>>(D.d_cheb, V.b, V.inv_diag, V.x, V.d, V.r,
                                                 V.d_coef, B->cs);
  } else {
    if ((st = apply32(V, D, V.x, V.t, s))) return st;
    kb_cheb_first<<<D.n_cheb, T256, 0, s>>>(D.d_cheb, V.b, V.t, V.inv_diag, V.x, V.d, V.r,
                                            V.d_coef, B->cs);
  }
  for (int j = 1; j < B->cheb_degree; ++j) {
    if ((st = apply32(V, D, V.d, V.t, s))) return st;
    kb_cheb_step<<<D.n_cheb, T256, 0, s>>>(D.d_cheb, V.t, V.inv_diag, V.x, V.d, V.r, V.d_coef,
                                           B->cs, j);
  }
  return cuda_status(cudaGetLastError(), "batch chebyshev");
}

// depth-0 x = V(b): descend every depth the plan's problems reach, all coarse
// solves, ascend
mfgb_status vcycle_b(const mfgb_batch *B, const Plan &P, cudaStream_t s) {
  size_t nd = 1;
  for (size_t l = 0; l < P.depth.size(); ++l)
    if (P.depth[l].n_cheb) nd = l + 2;  // depth l smooths, so depth l + 1 exists
  nd = std::min(nd, P.depth.size());
  mfgb_status st;
  for (size_t l = 0; l + 1 < nd; ++l) {
    const Depth &V = B->depth[l], &C = B->depth[l + 1];
    const DepthPlan &D = P.depth[l];
    if (!D.n_cheb) continue;
    if ((st = chebyshev_b(B, V, D, true, s))) return st;
    if ((st = apply32(V, D, V.x, V.t, s))) return st;
    kb_residual<<<D.n_cheb, T256, 0, s>>>(D.d_cheb, V.b, V.t, V.r);
    if ((st = cuda_status(cudaMemsetAsync(C.b, 0, sizeof(float) * C.n, s), "batch coarse b = 0")))
      return st;
    for (const PGroup &pg : D.pgroups) {
      const mfgb_operator *op = D.groups[pg.g];
      p_transfer<float>(true, op->n_cells, op->d_map, pg.map_c, V.r, V.inv_val, C.b, pg.P, s);
    }
    if (D.n_hcoarse)
      kb_h_restrict<<<D.n_hcoarse, T256, 0, s>>>(D.d_hcoarse, D.d_hp, V.r, C.b);
    if ((st = cuda_status(cudaGetLastError(), "batch restrict"))) return st;
  }
  if (P.n_coarse)
    kb_coarse<<<P.n_coarse, T256, P.coarse_smem, s>>>(P.d_coarse);
  if ((st = cuda_status(cudaGetLastError(), "batch coarse solves"))) return st;
  for (size_t l = nd - 1; l-- > 0;) {
    const Depth &V = B->depth[l], &C = B->depth[l + 1];
    const DepthPlan &D = P.depth[l];
    if (!D.n_cheb) continue;
    if (!D.pgroups.empty()) {
      if ((st = cuda_status(cudaMemsetAsync(V.t, 0, sizeof(float) * V.n, s), "batch t = 0")))
        return st;
      for (const PGroup &pg : D.pgroups) {
        const mfgb_operator *op = D.groups[pg.g];
        p_transfer<float>(false, op->n_cells, op->d_map, pg.map_c, C.x, nullptr, V.t, pg.P, s);
      }
      kb_add<<<D.n_pch, T256, 0, s>>>(D.d_pch, V.t, V.x);
    }
    if (D.n_hfine) kb_h_prolongate_add<<<D.n_hfine, T256, 0, s>>>(D.d_hfine, D.d_hp, C.x, V.x);
    if ((st = cuda_status(cudaGetLastError(), "batch prolongate"))) return st;
    if ((st = chebyshev_b(B, V, D, false, s))) return st;
  }
  return MFGB_OK;
}

// dst = M src (FP64 in and out)
mfgb_status precondition_b(const mfgb_batch *B, const Plan &P, double *dst, const double *src,
                           cudaStream_t s) {
  const Depth &V = B->depth[0];
  k_convert<float, double><<<grid1d(V.n), T256, 0, s>>>(V.n, src, V.b);
  mfgb_status st = vcycle_b(B, P, s);
  if (st) return st;
  k_convert<double, float><<<grid1d(V.n), T256, 0, s>>>(V.n, V.x, dst);
  return cuda_status(cudaGetLastError(), "batch precondition");
}

// A plan for the problems with active[i] != 0, gathered from the full plan:
// per part, contiguous segments of the union maps and geometric factors, of the
// identity-row list and of the coarse p-transfer maps are copied; chunk and
// transfer tables are rebuilt on the host.
mfgb_status gather_plan(const mfgb_batch *B, const std::vector<char> &active, Plan &out,
                        cudaStream_t s) {
  Plan P;
  P.owns = true;
  auto track = [&](void *m) { if (m) P.mem.push_back(m); };
  mfgb_status st = MFGB_OK;
  auto fail = [&](mfgb_status e) { free_plan(P); return e; };
  const size_t nd = B->depth.size();
  P.depth.resize(nd);
  // index of each problem's part per depth
  std::vector<std::vector<int>> part_at(B->n_problems, std::vector<int>(nd, -1));
  for (size_t l = 0; l < nd; ++l)
    for (size_t k = 0; k < B->depth[l].parts.size(); ++k)
      part_at[B->depth[l].parts[k].problem][l] = (int)k;
  for (size_t l = 0; l < nd; ++l) {
    const Depth &V = B->depth[l];
    const DepthPlan &F = B->full.depth[l];
    DepthPlan &D = P.depth[l];
    std::map<int, int> gidx;
    std::vector<int64_t> gcells;
    std::vector<std::vector<int>> gparts;
    int64_t n_cons = 0;
    for (size_t k = 0; k < V.parts.size(); ++k) {
      const Part &Q = V.parts[k];
      if (!active[Q.problem] || Q.group < 0) continue;
      auto it = gidx.find(Q.degree);
      if (it == gidx.end()) {
        it = gidx.emplace(Q.degree, (int)D.groups.size()).first;
        D.groups.push_back(union_shell(Q.degree, V.n));
        gcells.push_back(0);
        gparts.emplace_back();
      }
      gcells[it->second] += Q.n_cells;
      gparts[it->second].push_back((int)k);
      n_cons += Q.n_constrained;
    }
    int64_t *cons = nullptr;
    if ((st = dalloc((void **)&cons, sizeof(int64_t) * n_cons))) return fail(st);
    track(cons);
    D.d_cons = cons;
    D.n_cons = n_cons;
    int64_t cpos = 0;
    for (size_t g = 0; g < D.groups.size(); ++g) {
      mfgb_operator *op = D.groups[g];
      op->n_cells = gcells[g];
      const int64_t n3 = (int64_t)op->n * op->n * op->n;
      if ((st = dalloc((void **)&op->d_map, sizeof(uint32_t) * op->n_cells * n3)) ||
          (st = dalloc((void **)&op->d_G32, sizeof(float) * op->n_cells * 6 * n3)) ||
          (l == 0 && (st = dalloc((void **)&op->d_Gfx, sizeof(float2) * op->n_cells * 6 * n3))) ||
          (l == 0 && (st = dalloc((void **)&op->d_Gexp, sizeof(int) * op->n_cells))))
        return fail(st);
      int64_t c0 = 0;
      for (int k : gparts[g]) {
        const Part &Q = V.parts[k];
        const mfgb_operator *src = F.groups[Q.group];
        cudaMemcpyAsync(op->d_map + c0 * n3, src->d_map + Q.cell_off * n3,
                        sizeof(uint32_t) * Q.n_cells * n3, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(op->d_G32 + c0 * 6 * n3, src->d_G32 + Q.cell_off * 6 * n3,
                        sizeof(float) * Q.n_cells * 6 * n3, cudaMemcpyDeviceToDevice, s);
        if (l == 0) {
          cudaMemcpyAsync(op->d_Gfx + c0 * 6 * n3, src->d_Gfx + Q.cell_off * 6 * n3,
                          sizeof(float2) * Q.n_cells * 6 * n3, cudaMemcpyDeviceToDevice, s);
          cudaMemcpyAsync(op->d_Gexp + c0, src->d_Gexp + Q.cell_off, sizeof(int) * Q.n_cells,
                          cudaMemcpyDeviceToDevice, s);
        }
        cudaMemcpyAsync(cons + cpos, F.d_cons + Q.cons_off, sizeof(int64_t) * Q.n_constrained,
                        cudaMemcpyDeviceToDevice, s);
        cpos += Q.n_constrained;
        c0 += Q.n_cells;
      }
      // p-transfer group of this degree (same cells, same order)
      const PGroup *fpg = nullptr;
      for (const PGroup &q : F.pgroups)
        if (F.groups[q.g]->degree == op->degree) fpg = &q;
      if (fpg) {
        PGroup pg;
        pg.g = (int)g;
        pg.P = fpg->P;
        const int64_t nc3 = (int64_t)fpg->P.nc * fpg->P.nc * fpg->P.nc;
        if ((st = dalloc((void **)&pg.map_c, sizeof(uint32_t) * op->n_cells * nc3))) {
          return fail(st);
        }
        int64_t cc = 0;
        for (int k : gparts[g]) {
          const Part &Q = V.parts[k];
          cudaMemcpyAsync(pg.map_c + cc * nc3, fpg->map_c + Q.cell_off * nc3,
                          sizeof(uint32_t) * Q.n_cells * nc3, cudaMemcpyDeviceToDevice, s);
          cc += Q.n_cells;
        }
        D.pgroups.push_back(pg);
      }
    }
    // chunk and h-transfer tables
    std::vector<Chunk> cheb, pch, hfine, hcoarse;
    std::vector<HPart> hp;
    for (size_t k = 0; k < V.parts.size(); ++k) {
      const Part &Q = V.parts[k];
      if (!active[Q.problem] || Q.kind == 0) continue;
      append_chunks(cheb, Q.off, Q.n, (int)k);
      if (Q.kind == 1) append_chunks(pch, Q.off, Q.n, (int)k);
      if (Q.kind == 2) {
        const Part &R = B->depth[l + 1].parts[part_at[Q.problem][l + 1]];
        append_chunks(hfine, Q.off, Q.n, (int)hp.size());
        append_chunks(hcoarse, R.off, R.n, (int)hp.size());
        hp.push_back(HPart{hgrid(Q.box, Q.bs, R.box), Q.off, R.off});
      }
    }
    Chunk *c1 = nullptr, *c2 = nullptr, *c3 = nullptr, *c4 = nullptr;
    HPart *h1 = nullptr;
    if ((st = upload(&c1, cheb)) || (st = upload(&c2, pch)) || (st = upload(&c3, hfine)) ||
        (st = upload(&c4, hcoarse)) || (st = upload(&h1, hp)))
      return fail(st);
    track(c1); track(c2); track(c3); track(c4); track(h1);
    D.d_cheb = c1; D.n_cheb = (int)cheb.size();
    D.d_pch = c2; D.n_pch = (int)pch.size();
    D.d_hfine = c3; D.n_hfine = (int)hfine.size();
    D.d_hcoarse = c4; D.n_hcoarse = (int)hcoarse.size();
    D.d_hp = h1;
  }
  // coarse solves, outer CG tables
  std::vector<CoarseDesc> cd;
  std::vector<Chunk> all;
  std::vector<int> cbeg, pid;
  for (int i = 0; i < B->n_problems; ++i) {
    if (!active[i]) continue;
    cd.push_back(B->coarse_host[i]);
    const Part &Q = B->depth[0].parts[part_at[i][0]];
    cbeg.push_back((int)all.size());
    pid.push_back(i);
    append_chunks(all, Q.off, Q.n, part_at[i][0]);
    P.dofs += Q.n;
  }
  cbeg.push_back((int)all.size());
  CoarseDesc *dcd = nullptr;
  Chunk *dall = nullptr;
  int *dcb = nullptr, *dpid = nullptr;
  if ((st = upload(&dcd, cd)) || (st = upload(&dall, all)) || (st = upload(&dcb, cbeg)) ||
      (st = upload(&dpid, pid)))
    return fail(st);
  track(dcd); track(dall); track(dcb); track(dpid);
  P.d_coarse = dcd;
  P.n_coarse = (int)cd.size();
  P.coarse_smem = B->full.coarse_smem;
  P.d_all = dall;
  P.n_all = (int)all.size();
  P.d_cbeg = dcb;
  P.d_pid = dpid;
  P.n_prob = (int)pid.size();
  if ((st = cuda_status(cudaStreamSynchronize(s), "batch plan"))) return fail(st);
  out = P;
  return MFGB_OK;
}

mfgb_status check_params(const mfgb_box_desc *boxes, int n, const mfgb_mg_params *prm) {
  if (!boxes || n < 1 || !prm || prm->precision != 32 || prm->chebyshev_degree < 1 ||
      prm->chebyshev_degree > 32 || prm->smoothing_range <= 1.0 || prm->eig_iterations < 1 ||
      prm->coarse_cells < 1) {
    set_error("mfgb_batch_create: invalid argument (the batched V-cycle runs in FP32: precision 32)");
    return MFGB_ERR_INVALID_ARG;
  }
  for (int i = 0; i < n; ++i) {
    const mfgb_box_desc &b = boxes[i];
    if (b.degree < 1 || b.degree > 8 || b.nx < 1 || b.ny < 1 || b.nz < 1) {
      set_error("mfgb_batch_create: problem " + std::to_string(i) + ": degree 1..8 and cells >= 1");
      return MFGB_ERR_INVALID_ARG;
    }
  }
  return MFGB_OK;
}

mfgb_status build_batch(mfgb_batch *B, const mfgb_box_desc *boxes, int n,
                        const mfgb_mg_params *prm) {
  B->n_problems = n;
  B->cheb_degree = prm->chebyshev_degree;
  B->cs = 2 * prm->chebyshev_degree;
  B->boxes.assign(boxes, boxes + n);
  // ---- plan: parts per depth (problem order), offsets, union groups -------
  std::vector<std::vector<int>> part_at(n);  // part index per problem and depth
  for (int i = 0; i < n; ++i) {
    std::vector<mfgb_box_desc> lb;
    std::vector<int> kinds, strides;
    mg_plan_levels(boxes[i], prm->coarse_cells, lb, kinds, strides);
    if ((int64_t)B->depth.size() < (int64_t)lb.size()) B->depth.resize(lb.size());
    for (size_t l = 0; l < lb.size(); ++l) {
      Depth &D = B->depth[l];
      Part P;
      P.problem = i;
      P.box = lb[l];
      P.bs = BoxStride{{boxes[i].nx, boxes[i].ny, boxes[i].nz}, strides[l]};
      P.kind = kinds[l];
      P.degree = lb[l].degree;
      P.n = box_dofs(lb[l]);
      P.n_cells = (int64_t)lb[l].nx * lb[l].ny * lb[l].nz;
      P.n_constrained = box_boundary(lb[l]);
      P.off = D.n;
      D.n += P.n;
      part_at[i].push_back((int)D.parts.size());
      D.parts.push_back(P);
    }
  }
  for (auto &D : B->depth)
    if (D.n >= (int64_t)MFGB_INVALID_DOF) {
      set_error("mfgb_batch_create: a depth holds more DoFs than a 32-bit map can index");
      return MFGB_ERR_UNSUPPORTED;
    }
  mfgb_status st;
  for (size_t l = 0; l < B->depth.size(); ++l) {
    Depth &D = B->depth[l];
    std::map<int, int> gidx;  // degree -> group
    std::vector<int64_t> gcells;
    for (Part &P : D.parts) {
      if (l > 0 && P.kind == 0) continue;  // coarsest parts below depth 0 need no operator
      auto it = gidx.find(P.degree);
      if (it == gidx.end()) {
        it = gidx.emplace(P.degree, (int)D.groups.size()).first;
        D.groups.push_back(union_shell(P.degree, D.n));
        gcells.push_back(0);
      }
      P.group = it->second;
      P.cell_off = gcells[P.group];
      gcells[P.group] += P.n_cells;
      P.cons_off = D.n_cons;
      D.n_cons += P.n_constrained;
    }
    for (size_t g = 0; g < D.groups.size(); ++g) {
      mfgb_operator *op = D.groups[g];
      op->n_cells = gcells[g];
      const int64_t n3 = (int64_t)op->n * op->n * op->n;
      if ((st = dalloc((void **)&op->d_map, sizeof(uint32_t) * op->n_cells * n3)) ||
          (st = dalloc((void **)&op->d_G32, sizeof(float) * op->n_cells * 6 * n3)))
        return st;
      if (l == 0 && ((st = dalloc((void **)&op->d_Gfx, sizeof(float2) * op->n_cells * 6 * n3)) ||
                     (st = dalloc((void **)&op->d_Gexp, sizeof(int) * op->n_cells))))
        return st;
    }
    if ((st = dalloc((void **)&D.d_cons, sizeof(int64_t) * D.n_cons))) return st;
    float **vecs[] = {&D.x, &D.b, &D.r, &D.d, &D.t, &D.inv_diag, &D.inv_val};
    for (float **v : vecs)
      if ((st = dalloc((void **)v, sizeof(float) * D.n))) return st;
    if ((st = cuda_status(cudaMemset(D.inv_val, 0, sizeof(float) * D.n), "batch inv_val")))
      return st;
    // chunk tables
    std::vector<Chunk> cheb, pch, hfine, hcoarse;
    std::vector<HPart> hp;
    for (size_t k = 0; k < D.parts.size(); ++k) {
      const Part &P = D.parts[k];
      if (P.kind == 0) continue;
      append_chunks(cheb, P.off, P.n, (int)k);
      if (P.kind == 1) append_chunks(pch, P.off, P.n, (int)k);
      if (P.kind == 2) {
        const Part &Q = B->depth[l + 1].parts[part_at[P.problem][l + 1]];
        HPart h{hgrid(P.box, P.bs, Q.box), P.off, Q.off};
        append_chunks(hfine, P.off, P.n, (int)hp.size());
        append_chunks(hcoarse, Q.off, Q.n, (int)hp.size());
        hp.push_back(h);
      }
    }
    D.n_cheb = (int)cheb.size();
    D.n_pch = (int)pch.size();
    D.n_hfine = (int)hfine.size();
    D.n_hcoarse = (int)hcoarse.size();
    if ((st = upload(&D.d_cheb, cheb)) || (st = upload(&D.d_pch, pch)) ||
        (st = upload(&D.d_hfine, hfine)) || (st = upload(&D.d_hcoarse, hcoarse)) ||
        (st = upload(&D.d_hp, hp)))
      return st;
    // p-transfer groups: every part of a degree > 1 group goes to degree / 2
    for (size_t g = 0; g < D.groups.size(); ++g) {
      const int pf = D.groups[g]->degree;
      if (pf == 1 || l + 1 >= B->depth.size()) continue;
      PGroup pg;
      pg.g = (int)g;
      const int pc = std::max(1, pf / 2);
      mfgb_operator tmp_f, tmp_c;
      tmp_f.n = pf + 1;
      tmp_c.n = pc + 1;
      gll_nodes(tmp_f.n, tmp_f.gll_x, tmp_f.gll_w);
      gll_nodes(tmp_c.n, tmp_c.gll_x, tmp_c.gll_w);
      pg.P = ptransfer(&tmp_f, &tmp_c);
      const int64_t nc3 = (int64_t)tmp_c.n * tmp_c.n * tmp_c.n;
      if ((st = dalloc((void **)&pg.map_c, sizeof(uint32_t) * D.groups[g]->n_cells * nc3))) {
        D.pgroups.push_back(pg);
        return st;
      }
      D.pgroups.push_back(pg);
    }
  }
  // ---- outer CG tables -------------------------------------------------------
  {
    const Depth &D = B->depth[0];
    std::vector<Chunk> all;
    std::vector<int> cbeg;
    for (size_t k = 0; k < D.parts.size(); ++k) {
      cbeg.push_back((int)all.size());
      append_chunks(all, D.parts[k].off, D.parts[k].n, (int)k);
    }
    cbeg.push_back((int)all.size());
    B->n_all = (int)all.size();
    if ((st = upload(&B->d_all, all)) || (st = upload(&B->d_cbeg, cbeg))) return st;
    if ((st = dalloc((void **)&B->r, sizeof(double) * D.n)) ||
        (st = dalloc((void **)&B->z, sizeof(double) * D.n)) ||
        (st = dalloc((void **)&B->p, sizeof(double) * D.n)) ||
        (st = dalloc((void **)&B->v, sizeof(double) * D.n)) ||
        (st = dalloc((void **)&B->part, sizeof(double) * std::max(1, B->n_all))) ||
        (st = dalloc((void **)&B->d_scal, sizeof(BScal) * n)) ||
        (st = dalloc((void **)&B->d_active, sizeof(int))) ||
        (st = dalloc((void **)&B->d_active_dofs, sizeof(unsigned long long))) ||
        (st = dalloc((void **)&B->d_iter, sizeof(int))))
      return st;
    std::vector<int64_t> pd(n, 0);
    for (const Part &P : D.parts) pd[P.problem] = P.n;
    if ((st = upload(&B->d_pdofs, pd))) return st;
    if ((st = cuda_status(cudaMallocHost((void **)&B->h_active, sizeof(int)), "pinned flag")))
      return st;
  }
  // ---- per problem: its own hierarchy, copied into the batch, then freed ----
  std::vector<double> Ainv_all;
  std::vector<int32_t> cids_all;
  struct CoarseHost { int depth, part, nc; size_t a_off, id_off; };
  std::vector<CoarseHost> coarse_h;
  mfgb_mg_params p1 = *prm;
  for (int i = 0; i < n; ++i) {
    mfgb_mg *mg = nullptr;
    if ((st = mg_setup_without_lmax(&boxes[i], &p1, &mg))) return st;
    struct Guard { mfgb_mg *m; ~Guard() { mfgb_mg_destroy(m); } } guard{mg};
    if (mg->levels.size() != part_at[i].size()) {
      set_error("mfgb_batch_create: level plan mismatch");
      return MFGB_ERR_CUDA;
    }
    for (size_t l = 0; l < mg->levels.size(); ++l) {
      MgLevel &L = mg->levels[l];
      Depth &D = B->depth[l];
      Part &P = D.parts[part_at[i][l]];
      if (L.n != P.n || L.op->n_cells != P.n_cells || L.op->n_constrained != P.n_constrained) {
        set_error("mfgb_batch_create: level size mismatch");
        return MFGB_ERR_CUDA;
      }
      P.lmax = L.lmax;
      const int64_t n3 = (int64_t)L.op->n * L.op->n * L.op->n;
      if (P.group >= 0) {
        mfgb_operator *U = D.groups[P.group];
        kb_map_offset<<<grid1d(P.n_cells * n3), T256>>>(P.n_cells * n3, L.op->d_map,
                                                        U->d_map + P.cell_off * n3, (uint32_t)P.off);
        if ((st = cuda_status(cudaMemcpy(U->d_G32 + P.cell_off * 6 * n3, L.op->d_G32,
                                         sizeof(float) * P.n_cells * 6 * n3,
                                         cudaMemcpyDeviceToDevice),
                              "batch G32")))
          return st;
        if (l == 0) {
          // the outer FP64 operator: offset-accumulation kernel on per-cell scaled G
          if ((st = ensure_fx(L.op))) return st;
          if ((st = cuda_status(cudaMemcpy(U->d_Gfx + P.cell_off * 6 * n3, L.op->d_Gfx,
                                           sizeof(float2) * P.n_cells * 6 * n3,
                                           cudaMemcpyDeviceToDevice),
                                "batch Gfx")) ||
              (st = cuda_status(cudaMemcpy(U->d_Gexp + P.cell_off, L.op->d_Gexp,
                                           sizeof(int) * P.n_cells, cudaMemcpyDeviceToDevice),
                                "batch G exponents")))
            return st;
        }
        kb_offset_i64<<<grid1d(P.n_constrained), T256>>>(P.n_constrained, L.op->d_constrained,
                                                         D.d_cons + P.cons_off, P.off);
      }
      if ((st = cuda_status(cudaMemcpy(D.inv_diag + P.off, L.inv_diag, sizeof(float) * P.n,
                                       cudaMemcpyDeviceToDevice),
                            "batch inv_diag")))
        return st;
      if (P.kind == 1) {
        if ((st = cuda_status(cudaMemcpy(D.inv_val + P.off, L.inv_val, sizeof(float) * P.n,
                                         cudaMemcpyDeviceToDevice),
                              "batch inv_val")))
          return st;
        const MgLevel &Cl = mg->levels[l + 1];
        const Part &Q = B->depth[l + 1].parts[part_at[i][l + 1]];
        const int64_t nc3 = (int64_t)Cl.op->n * Cl.op->n * Cl.op->n;
        PGroup *pg = nullptr;
        for (auto &q : D.pgroups)
          if (q.g == P.group) pg = &q;
        if (!pg || pg->P.nc != Cl.op->n) {
          set_error("mfgb_batch_create: p-transfer group mismatch");
          return MFGB_ERR_CUDA;
        }
        kb_map_offset<<<grid1d(P.n_cells * nc3), T256>>>(P.n_cells * nc3, Cl.op->d_map,
                                                         pg->map_c + P.cell_off * nc3,
                                                         (uint32_t)Q.off);
      }
      if (P.kind == 0) {  // coarsest: FP64 inverse of the assembled interior matrix
        const int nc = mg->coarse.n;
        CoarseHost c{(int)l, part_at[i][l], nc, Ainv_all.size(), cids_all.size()};
        if (nc > 0) {
          if (nc > 1024) {
            set_error("mfgb_batch_create: coarse problem too large for a dense inverse");
            return MFGB_ERR_UNSUPPORTED;
          }
          std::vector<double> A((size_t)nc * nc), inv;
          std::vector<int64_t> ids(nc);
          if ((st = cuda_status(cudaMemcpy(A.data(), mg->coarse.A, sizeof(double) * A.size(),
                                           cudaMemcpyDeviceToHost),
                                "batch coarse A")) ||
              (st = cuda_status(cudaMemcpy(ids.data(), mg->coarse.ids, sizeof(int64_t) * nc,
                                           cudaMemcpyDeviceToHost),
                                "batch coarse ids")))
            return st;
          if (!spd_inverse(nc, A, inv)) {
            set_error("mfgb_batch_create: coarse matrix not positive definite");
            return MFGB_ERR_NONFINITE;
          }
          Ainv_all.insert(Ainv_all.end(), inv.begin(), inv.end());
          for (int64_t id : ids) cids_all.push_back((int32_t)id);
        }
        coarse_h.push_back(c);
      }
    }
    if ((st = cuda_status(cudaDeviceSynchronize(), "batch copy"))) return st;
  }
  // ---- lambda_max of every smoothed part: one power iteration per depth -----
  // over all its parts (the start, normalisation, FP32 operator, constrained
  // rows and Jacobi scaling of the single-problem estimate)
  for (size_t l = 0; l < B->depth.size(); ++l) {
    Depth &D = B->depth[l];
    if (!D.n_cheb) continue;
    const int np = (int)D.parts.size();
    std::vector<int64_t> poff(np);
    for (int k = 0; k < np; ++k) poff[k] = D.parts[k].off;
    int64_t *d_poff = nullptr;
    double *acc = nullptr;  // [2][np]: |v|^2, v.w
    if ((st = upload(&d_poff, poff)) || (st = dalloc((void **)&acc, sizeof(double) * 2 * np))) {
      cudaFree(d_poff);
      return st;
    }
    struct Free2 { void *a, *b; ~Free2() { cudaFree(a); cudaFree(b); } } f2{d_poff, acc};
    double *v = B->r, *w = B->z;  // depth-0-sized FP64 work vectors, free until the first solve
    DepthPlan DP;
    DP.groups = D.groups;
    DP.d_cons = D.d_cons;
    DP.n_cons = D.n_cons;
    if ((st = cuda_status(cudaMemset(D.t, 0, sizeof(float) * D.n), "batch lmax"))) return st;
    kb_pi_start<<<D.n_cheb, T256>>>(D.d_cheb, d_poff, v);
    if (D.n_cons) k_set_constrained<double><<<grid1d(D.n_cons), T256>>>(D.n_cons, D.d_cons, v, 0.0);
    for (int it = 0; it < prm->eig_iterations && !st; ++it) {
      cudaMemsetAsync(acc, 0, sizeof(double) * 2 * np, nullptr);
      kb_pi_dot<<<D.n_cheb, T256>>>(D.d_cheb, v, v, acc);
      kb_pi_normalize<<<D.n_cheb, T256>>>(D.d_cheb, acc, v, D.t);
      if ((st = apply32(D, DP, D.t, D.d, nullptr))) break;
      kb_pi_post<<<D.n_cheb, T256>>>(D.d_cheb, D.d, D.inv_diag, w);
      if (D.n_cons) k_set_constrained<double><<<grid1d(D.n_cons), T256>>>(D.n_cons, D.d_cons, w, 0.0);
      kb_pi_dot<<<D.n_cheb, T256>>>(D.d_cheb, v, w, acc + np);
      std::swap(v, w);
    }
    if (st) return st;
    std::vector<double> lam(np, 0.0);
    if ((st = cuda_status(cudaMemcpy(lam.data(), acc + np, sizeof(double) * np,
                                     cudaMemcpyDeviceToHost),
                          "batch lmax")))
      return st;
    for (int k = 0; k < np; ++k)
      if (D.parts[k].kind != 0) D.parts[k].lmax = 1.2 * lam[k];
  }
  // ---- Chebyshev coefficients per part (the single-problem recurrence) ------
  for (auto &D : B->depth) {
    std::vector<float> coef(D.parts.size() * B->cs, 0.f);
    for (size_t k = 0; k < D.parts.size(); ++k) {
      const Part &P = D.parts[k];
      if (P.kind == 0) continue;
      const double lmax = P.lmax, lmin = P.lmax / prm->smoothing_range;
      const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
      const double sigma = theta / delta;
      double rho = 1.0 / sigma;
      float *cf = coef.data() + k * B->cs;
      cf[0] = (float)(1.0 / theta);
      for (int j = 1; j < B->cheb_degree; ++j) {
        const double rho_new = 1.0 / (2.0 * sigma - rho);
        cf[2 * j - 1] = (float)(rho_new * rho);
        cf[2 * j] = (float)(2.0 * rho_new / delta);
        rho = rho_new;
      }
    }
    if ((st = upload(&D.d_coef, coef))) return st;
  }
  // ---- coarse descriptors ----------------------------------------------------
  if ((st = upload(&B->d_Ainv, Ainv_all)) || (st = upload(&B->d_cids, cids_all))) return st;
  std::vector<CoarseDesc> cd;
  int max_nc = 0;
  for (const auto &c : coarse_h) {
    const Depth &D = B->depth[c.depth];
    const Part &P = D.parts[c.part];
    CoarseDesc d{D.b + P.off, D.x + P.off, B->d_Ainv ? B->d_Ainv + c.a_off : nullptr,
                 B->d_cids ? B->d_cids + c.id_off : nullptr, c.nc, (int)P.n};
    cd.push_back(d);
    max_nc = std::max(max_nc, c.nc);
  }
  B->n_coarse = (int)cd.size();
  B->coarse_smem = (int)(sizeof(double) * std::max(1, max_nc));
  if ((st = upload(&B->d_coarse, cd))) return st;
  B->coarse_host.assign(n, CoarseDesc{});
  for (size_t k = 0; k < coarse_h.size(); ++k)
    B->coarse_host[B->depth[coarse_h[k].depth].parts[coarse_h[k].part].problem] = cd[k];
  // the full plan views the arrays above
  Plan &F = B->full;
  F.depth.resize(B->depth.size());
  for (size_t l = 0; l < B->depth.size(); ++l) {
    const Depth &D = B->depth[l];
    DepthPlan &P = F.depth[l];
    P.groups = D.groups;
    P.d_cons = D.d_cons;
    P.n_cons = D.n_cons;
    P.d_cheb = D.d_cheb; P.n_cheb = D.n_cheb;
    P.d_pch = D.d_pch; P.n_pch = D.n_pch;
    P.d_hfine = D.d_hfine; P.n_hfine = D.n_hfine;
    P.d_hcoarse = D.d_hcoarse; P.n_hcoarse = D.n_hcoarse;
    P.d_hp = D.d_hp;
    P.pgroups = D.pgroups;
  }
  std::vector<int> pid(n);
  for (int i = 0; i < n; ++i) pid[i] = i;
  if ((st = upload(&B->d_pid, pid))) return st;
  F.d_coarse = B->d_coarse;
  F.n_coarse = B->n_coarse;
  F.coarse_smem = B->coarse_smem;
  F.d_all = B->d_all;
  F.n_all = B->n_all;
  F.d_cbeg = B->d_cbeg;
  F.d_pid = B->d_pid;
  F.n_prob = n;
  F.dofs = B->depth[0].n;
  F.owns = false;
  return cuda_status(cudaDeviceSynchronize(), "batch set-up");
}

mfgb_status fork_stream(void *stream, cudaStream_t *s) {
  if (cudaStreamCreateWithFlags(s, cudaStreamNonBlocking) != cudaSuccess)
    return cuda_status(cudaErrorUnknown, "stream create");
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, (cudaStream_t)stream);
  cudaStreamWaitEvent(*s, ev, 0);
  cudaEventDestroy(ev);
  return MFGB_OK;
}

void join_stream(cudaStream_t s, void *stream) {
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, s);
  cudaStreamWaitEvent((cudaStream_t)stream, ev, 0);
  cudaEventDestroy(ev);
  cudaStreamDestroy(s);
}

}  // namespace
}  // namespace mfgb

using namespace mfgb;

extern "C" {

mfgb_status mfgb_batch_create(const mfgb_box_desc *boxes, int n_problems,
                              const mfgb_mg_params *params, mfgb_batch **out) {
  if (!out) {
    set_error("mfgb_batch_create: null output");
    return MFGB_ERR_INVALID_ARG;
  }
  *out = nullptr;
  mfgb_status st = check_params(boxes, n_problems, params);
  if (st) return st;
  mfgb_batch *B = new mfgb_batch();
  st = build_batch(B, boxes, n_problems, params);
  if (st) {
    cudaDeviceSynchronize();
    free_batch(B);
    return st;
  }
  *out = B;
  return MFGB_OK;
}

mfgb_status mfgb_batch_destroy(mfgb_batch *batch) {
  free_batch(batch);
  return MFGB_OK;
}

mfgb_status mfgb_batch_info(const mfgb_batch *B, int *n_problems, int64_t *h_offsets,
                            int *n_depths, int64_t *h_depth_dofs, int *h_levels) {
  if (!B) {
    set_error("mfgb_batch_info: null");
    return MFGB_ERR_INVALID_ARG;
  }
  if (n_problems) *n_problems = B->n_problems;
  if (n_depths) *n_depths = (int)B->depth.size();
  const Depth &D = B->depth[0];
  if (h_offsets) {
    for (size_t k = 0; k < D.parts.size(); ++k) h_offsets[k] = D.parts[k].off;
    h_offsets[D.parts.size()] = D.n;
  }
  if (h_depth_dofs)
    for (size_t l = 0; l < B->depth.size(); ++l) h_depth_dofs[l] = B->depth[l].n;
  if (h_levels) {
    for (int i = 0; i < B->n_problems; ++i) h_levels[i] = 0;
    for (const auto &Dl : B->depth)
      for (const auto &P : Dl.parts) h_levels[P.problem] += 1;
  }
  return MFGB_OK;
}

mfgb_status mfgb_batch_rhs_uniform(const mfgb_batch *B, const uint64_t *h_seeds, double *d_b,
                                   void *stream) {
  if (!B || !h_seeds || !d_b) {
    set_error("mfgb_batch_rhs_uniform: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  const Depth &D = B->depth[0];
  std::vector<double> h(D.n);
  for (const Part &P : D.parts) {
    std::mt19937_64 gen(h_seeds[P.problem]);
    double *b = h.data() + P.off;
    for (int64_t k = 0; k < P.n; ++k)
      b[k] = 2.0 * ((double)(gen() >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    // boundary DoFs (the box's constrained rows) are zero
    const int64_t X = (int64_t)P.degree * P.box.nx + 1, Y = (int64_t)P.degree * P.box.ny + 1,
                  Z = (int64_t)P.degree * P.box.nz + 1;
    for (int64_t z = 0; z < Z; ++z)
      for (int64_t y = 0; y < Y; ++y)
        for (int64_t x = 0; x < X; ++x)
          if (x == 0 || y == 0 || z == 0 || x == X - 1 || y == Y - 1 || z == Z - 1)
            b[x + X * (y + Y * z)] = 0.0;
  }
  cudaStream_t s = (cudaStream_t)stream;
  mfgb_status st = cuda_status(
      cudaMemcpyAsync(d_b, h.data(), sizeof(double) * D.n, cudaMemcpyHostToDevice, s), "batch rhs");
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(s), "batch rhs");
}

mfgb_status mfgb_batch_last_solve_stats(const mfgb_batch *B, int *n_replans) {
  if (!B || !n_replans) {
    set_error("mfgb_batch_last_solve_stats: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *n_replans = B->last_replans;
  return MFGB_OK;
}

mfgb_status mfgb_batch_last_solve_launches(const mfgb_batch *B, int *n_launches) {
  if (!B || !n_launches) {
    set_error("mfgb_batch_last_solve_launches: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *n_launches = B->last_launches;
  return MFGB_OK;
}

mfgb_status mfgb_batch_vmult(mfgb_batch *B, double *d_dst, const double *d_src, void *stream) {
  if (!B || !d_dst || !d_src || d_dst == d_src) {
    set_error("mfgb_batch_vmult: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  return apply64(B, B->full, d_src, d_dst, (cudaStream_t)stream);
}

mfgb_status mfgb_batch_precondition(mfgb_batch *B, double *d_dst, const double *d_src,
                                    void *stream) {
  if (!B || !d_dst || !d_src) {
    set_error("mfgb_batch_precondition: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  return precondition_b(B, B->full, d_dst, d_src, (cudaStream_t)stream);
}

// FP64 CG on every problem at once (deal.II SolverCG / ReductionControl per
// problem: tol_eff = max(tol, reduce |r0|)), the batched V-cycle as the
// preconditioner; one iteration of the batch = one CUDA graph launch.  When the
// problems still running hold at most 75 % of the current plan's DoFs, the
// plan is gathered again for them and the graph re-captured, so converged
// problems stop costing operator and V-cycle work.
mfgb_status mfgb_batch_cg_solve(mfgb_batch *B, const double *d_b, double *d_x,
                                const mfgb_cg_control *ctl, mfgb_solve_info *h_info,
                                void *stream) {
  if (!B || !d_b || !d_x || !ctl || !h_info || ctl->max_steps < 0) {
    set_error("mfgb_batch_cg_solve: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  cudaStream_t s = nullptr;
  mfgb_status st = fork_stream(stream, &s);
  if (st) return st;
  struct J { cudaStream_t s; void *o; ~J() { join_stream(s, o); } } join{s, stream};
  const int np = B->n_problems;
  const unsigned gp = (unsigned)((np + 127) / 128);
  const Plan &F = B->full;
  // r = b - A x; |r0|; z = M r; p = z; rz
  if ((st = apply64(B, F, d_x, B->v, s))) return st;
  kb_residual64<<<F.n_all, T256, 0, s>>>(F.d_all, d_b, B->v, B->r);
  kb_dot<<<F.n_all, T256, 0, s>>>(F.d_all, B->r, B->r, B->part);
  kb_init<<<np, T256, 0, s>>>(F.d_cbeg, F.d_pid, B->part, B->d_scal, ctl->tol, ctl->reduce);
  if ((st = precondition_b(B, F, B->z, B->r, s))) return st;
  kb_copy64<<<F.n_all, T256, 0, s>>>(F.d_all, B->z, B->p);
  kb_dot<<<F.n_all, T256, 0, s>>>(F.d_all, B->r, B->z, B->part);
  kb_sum_rz<<<np, T256, 0, s>>>(F.d_cbeg, F.d_pid, B->part, B->d_scal);
  kb_init_rz<<<gp, 128, 0, s>>>(np, B->d_scal);
  if ((st = cuda_status(cudaGetLastError(), "batch cg init"))) return st;
  std::vector<BScal> hs(np);
  auto read_scalars = [&]() {
    mfgb_status e = cuda_status(cudaMemcpyAsync(hs.data(), B->d_scal, sizeof(BScal) * np,
                                                cudaMemcpyDeviceToHost, s),
                                "batch cg scalars");
    if (!e) e = cuda_status(cudaStreamSynchronize(s), "batch cg scalars");
    return e;
  };
  if ((st = read_scalars())) return st;
  int running = 0;
  for (const BScal &q : hs) running += q.done == 0;

  // one CG iteration of the plan's problems, issued on s (in capture)
  auto iteration = [&](const Plan &P) -> mfgb_status {
    const int nb = P.n_prob;
    mfgb_status cap = apply64(B, P, B->p, B->v, s);
    if (!cap) {
      kb_dot<<<P.n_all, T256, 0, s>>>(P.d_all, B->p, B->v, B->part);
      kb_sum_pap<<<nb, T256, 0, s>>>(P.d_cbeg, P.d_pid, B->part, B->d_scal);
      kb_update<<<P.n_all, T256, 0, s>>>(P.d_all, d_x, B->r, B->p, B->v, B->d_scal, B->part);
      kb_zero_active<<<1, 1, 0, s>>>(B->d_active, B->d_active_dofs);
      kb_sum_check<<<nb, T256, 0, s>>>(P.d_cbeg, P.d_pid, B->part, B->d_scal, ctl->max_steps,
                                       B->d_active, B->d_pdofs, B->d_active_dofs);
      cap = precondition_b(B, P, B->z, B->r, s);
    }
    if (!cap) {
      kb_dot<<<P.n_all, T256, 0, s>>>(P.d_all, B->r, B->z, B->part);
      kb_sum_rz<<<nb, T256, 0, s>>>(P.d_cbeg, P.d_pid, B->part, B->d_scal);
      kb_direction<<<P.n_all, T256, 0, s>>>(P.d_all, B->z, B->p, B->d_scal);
      kb_roll<<<gp, 128, 0, s>>>(np, B->d_scal);
    }
    return cap;
  };
  // The plan's iterations as one graph: a conditional while node whose body is
  // one iteration plus the condition kernel (kb_continue), so one launch runs
  // until every problem is done, the running problems hold at most 75 % of the
  // plan's DoFs, or max_steps iterations (device-side loop; the host only
  // gathers new plans).  Where the body cannot be built as a conditional graph
  // the plan falls back to one graph launch per iteration (*looped = false).
  auto capture = [&](const Plan &P, cudaGraphExec_t *exec, bool *looped) -> mfgb_status {
    mfgb_status e;
    *looped = false;
    {
      cudaGraph_t graph = nullptr;
      cudaGraphConditionalHandle h;
      cudaGraphNodeParams cp{};
      cudaGraphNode_t node;
      bool ok = cudaGraphCreate(&graph, 0) == cudaSuccess &&
                cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault) ==
                    cudaSuccess;
      if (ok) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        ok = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess;
      }
      if (ok) {
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
          mfgb_status cap = iteration(P);
          const unsigned long long threshold = (unsigned long long)(0.75 * (double)P.dofs);
          if (!cap)
            kb_continue<<<1, 1, 0, s>>>(h, B->d_active, B->d_active_dofs, threshold, B->d_iter,
                                        ctl->max_steps);
          cudaGraph_t out = nullptr;
          const cudaError_t ce = cudaStreamEndCapture(s, &out);
          if (cap) {
            cudaGraphDestroy(graph);
            return cap;
          }
          ok = ce == cudaSuccess && cudaGraphInstantiate(exec, graph, 0) == cudaSuccess;
        }
      }
      if (graph) cudaGraphDestroy(graph);
      if (ok) {
        *looped = true;
        return MFGB_OK;
      }
      cudaGetLastError();
      *exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    if ((e = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture")))
      return e;
    mfgb_status cap = iteration(P);
    if (!cap)
      cudaMemcpyAsync(B->h_active, B->d_active, sizeof(int), cudaMemcpyDeviceToHost, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (cap) {
      if (graph) cudaGraphDestroy(graph);
      return cap;
    }
    if ((e = cuda_status(ce, "end capture"))) return e;
    e = cuda_status(cudaGraphInstantiate(exec, graph, 0), "instantiate");
    cudaGraphDestroy(graph);
    return e;
  };

  Plan sub;  // the gathered plan in use (owns its arrays), when not the full one
  struct FreeSub { Plan *p; ~FreeSub() { free_plan(*p); } } free_sub{&sub};
  const Plan *cur = &F;
  B->last_replans = 0;
  B->last_launches = 0;
  if (running > 0 && ctl->max_steps > 0) {
    cudaGraphExec_t exec = nullptr;
    bool looped = false;
    if ((st = capture(*cur, &exec, &looped))) return st;
    for (int it = 0; it < ctl->max_steps; ++it) {
      cudaError_t e = cudaSuccess;
      if (looped) e = cudaMemsetAsync(B->d_iter, 0, sizeof(int), s);
      if (e == cudaSuccess) e = cudaGraphLaunch(exec, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      ++B->last_launches;
      if (e != cudaSuccess) {
        st = cuda_status(e, "batch cg iteration");
        break;
      }
      if ((st = read_scalars())) break;
      std::vector<char> active(np, 0);
      int64_t dofs = 0;
      int n_run = 0;
      for (int i = 0; i < np; ++i)
        if (!hs[i].done) {
          active[i] = 1;
          ++n_run;
          dofs += B->depth[0].parts[i].n;
        }
      if (n_run == 0) break;
      // re-plan for the running problems once they hold <= 75 % of the plan's DoFs
      if (dofs <= 0.75 * (double)cur->dofs) {
        Plan next;
        if ((st = gather_plan(B, active, next, s))) break;
        cudaGraphExecDestroy(exec);
        exec = nullptr;
        free_plan(sub);
        sub = next;
        cur = &sub;
        ++B->last_replans;
        if ((st = capture(*cur, &exec, &looped))) break;
      }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (st) return st;
  }
  if ((st = read_scalars())) return st;
  if ((st = mfgb_check_device_errors(s))) return st;
  int failed = 0, nonfinite = 0;
  for (int i = 0; i < np; ++i) {
    h_info[i].steps = hs[i].its;
    h_info[i].initial = hs[i].res0;
    h_info[i].last = hs[i].res;
    h_info[i].converged = hs[i].done == 1;
    failed += hs[i].done != 1;
    nonfinite += std::isnan(hs[i].res);
  }
  if (nonfinite) {
    set_error("mfgb_batch_cg_solve: NaN residual in " + std::to_string(nonfinite) + " problem(s)");
    return MFGB_ERR_NONFINITE;
  }
  if (failed) {
    set_error("mfgb_batch_cg_solve: " + std::to_string(failed) + " problem(s) reached max_steps");
    return MFGB_ERR_NOT_CONVERGED;
  }
  return MFGB_OK;
}

}  // extern "C"
