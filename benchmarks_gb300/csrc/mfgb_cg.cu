// mfgb_cg.cu -- conjugate gradients on the BK5 operator.
//
// Semantics of deal.II SolverCG with ReductionControl as used by the reference
// (bp5_kokkos/benchmark.cc:355-378; bakeoff_problems_dealii/tests/
// scaling_bp35_kokkos_kernel/program.cc:263-287): r0 = b - A x0,
// tol_eff = max(tol, reduce * |r0|), success as soon as |r_k| <= tol_eff,
// failure when k reaches max_steps.  Preconditioner: identity or the inverse
// diagonal (DiagonalMatrix).
//
// GB300 layout of one iteration (all on the device, no host round trip):
//   1. bk5 apply  v += A p (cell loop)
//   2. constrained rows v_c = p_c
//   3. p.v        per-CTA partials (one read of p and v)
//   4. update     alpha = rz / pAp; x += alpha p; r -= alpha v;
//                 partials of r.r and r.z (z = Dinv r, never stored)
//   5. direction  |r| test -> done flag; beta; p = z + beta p; v = 0
// Each kernel returns at once when the done flag is set, so a CUDA graph of
// K iterations can be replayed until the host sees the flag.  All reductions
// are two-stage with a fixed order (deterministic).
#include <cmath>
#include <vector>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"

namespace mfgb {

struct CgScalars {
  double rz[2];     // r.z of the current direction, by iteration parity
  double res[2];    // residual norm, by parity
  int its[2];       // completed iterations, by parity
  double tol_eff;
  int max_steps;
  int done;         // 0 running, 1 converged, 2 failed
  int final_its;
  double final_res;
  int loop_runs;    // body runs of the device-side loop (mfgb_cg_solve)
};

// condition of the device-side solve loop: repeat the captured block of
// iterations while the solve runs, at most max_runs times (a hard bound; the
// done flag is set at max_steps anyway)
__global__ void cg_continue_kernel(cudaGraphConditionalHandle h, CgScalars *sc, int max_runs) {
  const int r = sc->loop_runs + 1;
  sc->loop_runs = r;
  cudaGraphSetConditional(h, (!sc->done && r < max_runs) ? 1u : 0u);
}

constexpr int VEC_THREADS = 256;
constexpr int VEC_BLOCKS = 152 * 8;

template <int T>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < T / 32; ++i) s += sh[i];
  return s;  // valid in thread 0
}

// every CTA sums the same partials in the same order -> identical result
__device__ __forceinline__ double sum_partials(const double *__restrict__ p, int n, int stride,
                                               double *sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += p[(size_t)i * stride];
  double s = block_sum<VEC_THREADS>(v, sh);
  __syncthreads();
  if (threadIdx.x == 0) sh[32] = s;
  __syncthreads();
  return sh[32];
}

// identity rows of the constrained DoFs: v_c = p_c (many CTAs)
__global__ void __launch_bounds__(VEC_THREADS)
    cg_constrained_copy_kernel(int64_t nc, const int64_t *__restrict__ c,
                               const double *__restrict__ p, double *__restrict__ v,
                               const CgScalars *__restrict__ sc) {
  if (sc->done) return;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nc;
       t += (int64_t)gridDim.x * blockDim.x)
    v[c[t]] = p[c[t]];
}

// per-CTA partials of p.v (v = A p including the identity rows)
__global__ void __launch_bounds__(VEC_THREADS)
    cg_dot_pv_kernel(int64_t n, const double *__restrict__ p, const double *__restrict__ v,
                     double *__restrict__ partials, const CgScalars *__restrict__ sc) {
  if (sc->done) return;
  __shared__ double sh[40];
  double s = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    s = __fma_rn(p[t], v[t], s);
  const double bs = block_sum<VEC_THREADS>(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bs;
}

__global__ void __launch_bounds__(VEC_THREADS)
    cg_update_kernel(int64_t n, double *__restrict__ x, double *__restrict__ r,
                     const double *__restrict__ p, const double *__restrict__ v,
                     const double *__restrict__ dinv, const double *__restrict__ pap_partials,
                     int n_pap, double *__restrict__ out_partials, CgScalars *__restrict__ sc,
                     int parity) {
  if (sc->done) return;
  __shared__ double sh[40];
  const double pap = sum_partials(pap_partials, n_pap, 1, sh);
  const double alpha = sc->rz[parity] / pap;
  double rr = 0.0, rz = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double pt = p[t];
    x[t] = __fma_rn(alpha, pt, x[t]);
    const double rt = __fma_rn(-alpha, v[t], r[t]);
    r[t] = rt;
    const double zt = dinv ? dinv[t] * rt : rt;
    rr = __fma_rn(rt, rt, rr);
    rz = __fma_rn(rt, zt, rz);
  }
  const double srr = block_sum<VEC_THREADS>(rr, sh);
  __syncthreads();
  const double srz = block_sum<VEC_THREADS>(rz, sh);
  if (threadIdx.x == 0) {
    out_partials[2 * blockIdx.x] = srr;
    out_partials[2 * blockIdx.x + 1] = srz;
  }
}

__global__ void __launch_bounds__(VEC_THREADS)
    cg_direction_kernel(int64_t n, const double *__restrict__ r, double *__restrict__ p,
                        double *__restrict__ v, const double *__restrict__ dinv,
                        const double *__restrict__ partials, int n_part,
                        CgScalars *__restrict__ sc, int parity) {
  if (sc->done) return;
  __shared__ double sh[40];
  const double rr = sum_partials(partials, n_part, 2, sh);
  const double rz_new = sum_partials(partials + 1, n_part, 2, sh);
  const double res = sqrt(rr);
  const int it = sc->its[parity] + 1;
  const bool converged = res <= sc->tol_eff;
  const bool failed = !converged && (it >= sc->max_steps || isnan(res));
  if (converged || failed) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      sc->final_its = it;
      sc->final_res = res;
      sc->done = converged ? 1 : 2;
    }
    return;
  }
  const double beta = rz_new / sc->rz[parity];
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double rt = r[t];
    const double zt = dinv ? dinv[t] * rt : rt;
    p[t] = __fma_rn(beta, p[t], zt);
    v[t] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->rz[parity ^ 1] = rz_new;
    sc->its[parity ^ 1] = it;
    sc->res[parity ^ 1] = res;
  }
}

// r = b - v; z = Dinv r; p = z; partials of r.r and r.z
__global__ void __launch_bounds__(VEC_THREADS)
    cg_init_kernel(int64_t n, const double *__restrict__ b, const double *__restrict__ v,
                   double *__restrict__ r, double *__restrict__ p, const double *__restrict__ dinv,
                   double *__restrict__ out_partials) {
  __shared__ double sh[40];
  double rr = 0.0, rz = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double rt = b[t] - v[t];
    r[t] = rt;
    const double zt = dinv ? dinv[t] * rt : rt;
    p[t] = zt;
    rr = __fma_rn(rt, rt, rr);
    rz = __fma_rn(rt, zt, rz);
  }
  const double srr = block_sum<VEC_THREADS>(rr, sh);
  __syncthreads();
  const double srz = block_sum<VEC_THREADS>(rz, sh);
  if (threadIdx.x == 0) {
    out_partials[2 * blockIdx.x] = srr;
    out_partials[2 * blockIdx.x + 1] = srz;
  }
}

__global__ void __launch_bounds__(VEC_THREADS)
    dot_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
               double *__restrict__ partials) {
  __shared__ double sh[40];
  double s = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    s = __fma_rn(a[t], b[t], s);
  const double bs = block_sum<VEC_THREADS>(s, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = bs;
}

__global__ void finish_sum_kernel(const double *__restrict__ partials, int n, int stride,
                                  double *__restrict__ out) {
  __shared__ double sh[40];
  const double s = sum_partials(partials, n, stride, sh);
  if (threadIdx.x == 0) *out = s;
}

int dot_partials_count() { return VEC_BLOCKS; }

// a.b into device memory (*out), stream ordered, no host synchronisation;
// partials holds dot_partials_count() doubles
cudaError_t dot_to_device(int64_t n, const double *a, const double *b, double *partials,
                          double *out, cudaStream_t s) {
  dot_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, a, b, partials);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(partials, VEC_BLOCKS, 1, out);
  return cudaGetLastError();
}

}  // namespace mfgb

using namespace mfgb;

namespace {

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

mfgb_status alloc(DevBuf &b, size_t bytes) {
  if (alloc_hook_fails("cg work vector")) return MFGB_ERR_OUT_OF_MEMORY;
  const cudaError_t e = cudaMalloc(&b.p, bytes);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    set_error("cudaMalloc failed (out of device memory)");
    return MFGB_ERR_OUT_OF_MEMORY;
  }
  return cuda_status(e, "cudaMalloc");
}

}  // namespace

extern "C" mfgb_status mfgb_dot(int64_t n, const double *d_a, const double *d_b, double *h_result,
                                void *stream) {
  if (n < 0 || (n > 0 && (!d_a || !d_b)) || !h_result) {
    set_error("mfgb_dot: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  DevBuf part;
  mfgb_status st = alloc(part, sizeof(double) * (VEC_BLOCKS + 1));
  if (st) return st;
  double *pp = (double *)part.p;
  dot_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, d_a, d_b, pp);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(pp, VEC_BLOCKS, 1, pp + VEC_BLOCKS);
  st = cuda_status(cudaMemcpyAsync(h_result, pp + VEC_BLOCKS, sizeof(double),
                                   cudaMemcpyDeviceToHost, s),
                   "dot copy");
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(s), "dot sync");
}

extern "C" mfgb_status mfgb_cg_solve(const mfgb_operator *cop, const double *d_b, double *d_x,
                                     const double *d_inv_diag, const mfgb_cg_control *ctl,
                                     mfgb_solve_info *info, void *stream) {
  if (!cop || !d_b || !d_x || !ctl || !info || ctl->max_steps < 0) {
    set_error("mfgb_cg_solve: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (ctl->arith != MFGB_ARITH_FP64 && ctl->arith != MFGB_ARITH_FP64_DF) {
    set_error("mfgb_cg_solve: unknown arith");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb_operator *op = const_cast<mfgb_operator *>(cop);
  const int64_t n = op->n_dofs;
  cudaStream_t user = (cudaStream_t)stream;
  mfgb_status st;
  if ((st = ensure_arith(op, ctl->arith))) return st;

  // work vectors: r, p, v, partials, scalars
  DevBuf br, bp, bv, bpart, bsc;
  if ((st = alloc(br, sizeof(double) * n)) || (st = alloc(bp, sizeof(double) * n)) ||
      (st = alloc(bv, sizeof(double) * n)))
    return st;
  double *r = (double *)br.p, *p = (double *)bp.p, *v = (double *)bv.p;
  const double *dinv = d_inv_diag;
  constexpr int PAP_CAP = 152 * 64 + 1;
  if ((st = alloc(bpart, sizeof(double) * (PAP_CAP + 2 * VEC_BLOCKS + 8)))) return st;
  double *pap_part = (double *)bpart.p;
  double *vec_part = pap_part + PAP_CAP;
  if ((st = alloc(bsc, sizeof(CgScalars)))) return st;
  CgScalars *sc = (CgScalars *)bsc.p;

  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return cuda_status(cudaErrorUnknown, "stream create");
  }
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{s};
  cudaEvent_t ev;
  cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  cudaEventRecord(ev, user);
  cudaStreamWaitEvent(s, ev, 0);
  cudaEventDestroy(ev);

  // r0 = b - A x0, p0 = z0
  if ((st = vmult_impl(op, v, d_x, ctl->arith, nullptr, nullptr, s))) return st;
  cg_init_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, d_b, v, r, p, dinv, vec_part);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(vec_part, VEC_BLOCKS, 2, vec_part + 2 * VEC_BLOCKS);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(vec_part + 1, VEC_BLOCKS, 2,
                                              vec_part + 2 * VEC_BLOCKS + 1);
  double h2[2];
  if ((st = cuda_status(cudaMemcpyAsync(h2, vec_part + 2 * VEC_BLOCKS, 2 * sizeof(double),
                                        cudaMemcpyDeviceToHost, s),
                        "cg init copy")))
    return st;
  if ((st = cuda_status(cudaStreamSynchronize(s), "cg init"))) return st;
  const double res0 = std::sqrt(h2[0]);
  info->initial = res0;
  info->last = res0;
  info->steps = 0;
  info->converged = 0;
  const double tol_eff = std::fmax(ctl->tol, ctl->reduce * res0);
  if (res0 <= tol_eff) {
    info->converged = 1;
    return MFGB_OK;
  }
  if (std::isnan(res0)) {
    set_error("mfgb_cg_solve: initial residual is NaN");
    return MFGB_ERR_NONFINITE;
  }
  if (ctl->max_steps == 0) return MFGB_ERR_NOT_CONVERGED;

  CgScalars hsc{};
  hsc.rz[0] = h2[1];
  hsc.res[0] = res0;
  hsc.its[0] = 0;
  hsc.tol_eff = tol_eff;
  hsc.max_steps = ctl->max_steps;
  hsc.done = 0;
  if ((st = cuda_status(cudaMemcpyAsync(sc, &hsc, sizeof(hsc), cudaMemcpyHostToDevice, s),
                        "cg scalars")))
    return st;
  if ((st = cuda_status(cudaMemsetAsync(v, 0, sizeof(double) * n, s), "v = 0"))) return st;

  // K iterations (parity alternates, K even) captured as the body of a
  // conditional while node: one graph launch runs the whole solve on the device
  // (cg_continue_kernel ends it once the done flag is set).  Where the driver
  // cannot build that graph, the K iterations form a plain graph the host
  // relaunches until done.
  const int K = 16;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool looped = false;
  // capture the K iterations into `graph` (as the body of a while node when
  // try_loop) and instantiate it
  auto build = [&](bool try_loop) -> mfgb_status {
    mfgb_status bst;
    graph = nullptr;
    exec = nullptr;
    looped = false;
    cudaGraphConditionalHandle cond_h{};
    if (try_loop) {
      cudaGraphNodeParams cp{};
      cudaGraphNode_t node;
      looped = cudaGraphCreate(&graph, 0) == cudaSuccess &&
               cudaGraphConditionalHandleCreate(&cond_h, graph, 1, cudaGraphCondAssignDefault) ==
                   cudaSuccess;
      if (looped) {
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond_h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        looped = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp) == cudaSuccess &&
                 cudaStreamBeginCaptureToGraph(s, cp.conditional.phGraph_out[0], nullptr, nullptr,
                                               0, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      }
      if (!looped) {
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        graph = nullptr;
        return MFGB_ERR_UNSUPPORTED;
      }
    } else if ((bst = cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                                  "begin capture"))) {
      return bst;
    }
    mfgb_status cap_st = MFGB_OK;
    for (int k = 0; k < K && cap_st == MFGB_OK; ++k) {
      const int parity = k & 1;
      cap_st = apply_add_impl(op, v, p, ctl->arith, s, &sc->done);
      if (cap_st) break;
      if (op->n_constrained)
        cg_constrained_copy_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(op->n_constrained,
                                                                      op->d_constrained, p, v, sc);
      cg_dot_pv_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, p, v, pap_part, sc);
      cg_update_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, d_x, r, p, v, dinv, pap_part,
                                                          VEC_BLOCKS, vec_part, sc, parity);
      cg_direction_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, r, p, v, dinv, vec_part,
                                                             VEC_BLOCKS, sc, parity);
    }
    if (looped && !cap_st)
      cg_continue_kernel<<<1, 1, 0, s>>>(cond_h, sc, ctl->max_steps / K + 2);
    cudaGraph_t captured = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &captured);
    if (!looped) graph = captured;
    if (!cap_st) cap_st = cuda_status(ce, "end capture");
    if (!cap_st) cap_st = cuda_status(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
    if (cap_st) {
      if (graph) cudaGraphDestroy(graph);
      graph = nullptr;
      exec = nullptr;
    }
    return cap_st;
  };
  if (build(true) && (st = build(false))) return st;
  CgScalars out{};
  for (;;) {
    cudaError_t e = cudaGraphLaunch(exec, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&out, sc, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      return cuda_status(e, "cg iterations");
    }
    if (out.done) break;
  }
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  info->steps = out.final_its;
  info->last = out.final_res;
  info->converged = out.done == 1;
  if ((st = mfgb_check_device_errors(s))) return st;
  if (out.done == 1) return MFGB_OK;
  if (std::isnan(out.final_res)) {
    set_error("mfgb_cg_solve: residual became NaN");
    return MFGB_ERR_NONFINITE;
  }
  set_error("mfgb_cg_solve: max_steps reached");
  return MFGB_ERR_NOT_CONVERGED;
}

// ---------------------------------------------------------------------------
// Conjugate gradients without any device allocation.
//
// For callers that must not allocate device memory while solving: code that
// runs under an external memory budget or a pool it does not own (a host
// application whose allocator reserved the device, a solver called from inside
// another library's time step), and code paths where a cudaMalloc could block
// or fail at a bad moment.  The work vectors, the reduction partials and the
// device scalars live in one file-scope __device__ array, sized for at most
// MFGB_CG_NOALLOC_MAX_DOFS unknowns (about 25 MB).  Every GPU that loads this
// library keeps that array until the process exits.  Every call shares it and
// it keeps the previous call's contents, so everything the solve reads is
// initialised by the solve itself; calls whose work overlaps on the GPU (two
// streams, two host threads on one device) race on it and must be serialised
// by the caller.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress, once per device); make that first call before
// any stream capture.
// ---------------------------------------------------------------------------
#include <mutex>

namespace mfgb {

constexpr int64_t NOALLOC_PAP_CAP = 152 * 64 + 1;
constexpr int64_t NOALLOC_VEC_PART = 2 * VEC_BLOCKS + 8;
constexpr int64_t NOALLOC_SCALARS = 32;  // doubles reserved for CgScalars
// the last 8 bytes of the scalar slot hold the double-float range check's int
static_assert(sizeof(CgScalars) <= NOALLOC_SCALARS * sizeof(double) - 8, "scalar slot too small");
constexpr int64_t NOALLOC_DOUBLES =
    3 * (int64_t)MFGB_CG_NOALLOC_MAX_DOFS + NOALLOC_PAP_CAP + NOALLOC_VEC_PART + NOALLOC_SCALARS;

static __device__ __align__(256) double g_cg_noalloc_scratch[NOALLOC_DOUBLES];

static std::mutex g_noalloc_mutex;
static double *g_noalloc_ptr[64] = {nullptr};

// device address of the scratch array on the current device (looked up once
// per device and cached for the life of the process; a cudaDeviceReset or a
// teardown of the primary context invalidates the cached address, so the
// library must not be used across either)
static mfgb_status noalloc_scratch(double **out) {
  int dev = 0;
  mfgb_status st = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
  if (st) return st;
  if (dev < 0 || dev >= 64) {
    set_error("mfgb_cg_solve_noalloc: device ordinal above 63");
    return MFGB_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_cg_noalloc_scratch), "cudaGetSymbolAddress");
    if (st) return st;
    g_noalloc_ptr[dev] = (double *)p;
  }
  *out = g_noalloc_ptr[dev];
  return MFGB_OK;
}

// vmult (partials == nullptr) or accumulate-with-energy, never allocating:
// double-float arithmetic uses the operator's split copy of G when an earlier
// call created it, and otherwise splits the FP64 geometric factors on load.
// The double-float kernels without per-cell scaling also check src's range
// into the device error word (range_slot: an int of the scratch array).
static mfgb_status noalloc_apply(const mfgb_operator *op, double *dst, const double *src, int arith,
                                 double *partials, int *grid, cudaStream_t s, const int *done,
                                 int *range_slot, bool accumulate = false) {
  mfgb_status st;
  const bool full = !partials && !accumulate;
  if (full && (st = cuda_status(cudaMemsetAsync(dst, 0, sizeof(double) * op->n_dofs, s),
                                "dst = 0")))
    return st;
  if (arith == MFGB_ARITH_FP64_DF && !(op->d_Gfx && !partials) &&
      (st = vec_range_check(range_slot, op->n_dofs, src, s)))
    return st;
  cudaError_t e;
  if (arith == MFGB_ARITH_FP64)
    e = bk5_f64(op->n, op->n_cells, op->d_map, op->d_G, src, dst, op->D, partials, grid, s, done);
  else if (op->d_Gfx && !partials)
    e = bk5_fx(op->n, op->n_cells, op->d_map, op->d_Gfx, op->d_Gexp, src, dst, op->D, s, done);
  else if (op->d_Gdf)
    e = bk5_df(op->n, op->n_cells, op->d_map, op->d_Gdf, src, dst, op->D, partials, grid, s, done);
  else
    e = bk5_df_g64(op->n, op->n_cells, op->d_map, op->d_G, src, dst, op->D, s, done);
  if ((st = cuda_status(e, "bk5 kernel"))) return st;
  if (full)
    return cuda_status(copy_constrained(op->n_constrained, op->d_constrained, src, dst, s),
                       "constrained rows");
  return MFGB_OK;
}

}  // namespace mfgb

extern "C" mfgb_status mfgb_cg_solve_noalloc(const mfgb_operator *op, const double *d_b,
                                             double *d_x, const double *d_inv_diag,
                                             const mfgb_cg_control *ctl, mfgb_solve_info *info,
                                             void *stream) {
  if (!op || !d_b || !d_x || !ctl || !info || ctl->max_steps < 0) {
    set_error("mfgb_cg_solve_noalloc: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (ctl->arith != MFGB_ARITH_FP64 && ctl->arith != MFGB_ARITH_FP64_DF) {
    set_error("mfgb_cg_solve_noalloc: unknown arith");
    return MFGB_ERR_INVALID_ARG;
  }
  if (op->quadrature != 0) {
    set_error("mfgb_cg_solve_noalloc: GLL-collocated operators only (use mfgb_cg_solve)");
    return MFGB_ERR_UNSUPPORTED;
  }
  const int64_t n = op->n_dofs;
  if (n > (int64_t)MFGB_CG_NOALLOC_MAX_DOFS) {
    set_error("mfgb_cg_solve_noalloc: " + std::to_string(n) + " DoFs exceed the fixed scratch of " +
              std::to_string((long long)MFGB_CG_NOALLOC_MAX_DOFS) +
              " DoFs; use mfgb_cg_solve for larger problems");
    return MFGB_ERR_UNSUPPORTED;
  }
  double *scratch = nullptr;
  mfgb_status st = noalloc_scratch(&scratch);
  if (st) return st;
  double *r = scratch;
  double *p = r + MFGB_CG_NOALLOC_MAX_DOFS;
  double *v = p + MFGB_CG_NOALLOC_MAX_DOFS;
  double *pap_part = v + MFGB_CG_NOALLOC_MAX_DOFS;
  double *vec_part = pap_part + NOALLOC_PAP_CAP;
  CgScalars *sc = (CgScalars *)(vec_part + NOALLOC_VEC_PART);
  int *range_slot = reinterpret_cast<int *>(vec_part + NOALLOC_VEC_PART + NOALLOC_SCALARS - 1);
  cudaStream_t s = (cudaStream_t)stream;
  const double *dinv = d_inv_diag;
  // double-float without a prebuilt copy of G splits the FP64 factors on load:
  // their per-cell range goes to the device error word
  if (ctl->arith == MFGB_ARITH_FP64_DF && !op->d_Gfx && !op->d_Gdf &&
      (st = cells_range_check(op->n_cells, 6 * op->n * op->n * op->n, op->d_G, s)))
    return st;

  // r0 = b - A x0, p0 = z0
  if ((st = noalloc_apply(op, v, d_x, ctl->arith, nullptr, nullptr, s, nullptr, range_slot)))
    return st;
  cg_init_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, d_b, v, r, p, dinv, vec_part);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(vec_part, VEC_BLOCKS, 2, vec_part + 2 * VEC_BLOCKS);
  finish_sum_kernel<<<1, VEC_THREADS, 0, s>>>(vec_part + 1, VEC_BLOCKS, 2,
                                              vec_part + 2 * VEC_BLOCKS + 1);
  double h2[2];
  if ((st = cuda_status(cudaMemcpyAsync(h2, vec_part + 2 * VEC_BLOCKS, 2 * sizeof(double),
                                        cudaMemcpyDeviceToHost, s),
                        "cg init copy")) ||
      (st = cuda_status(cudaStreamSynchronize(s), "cg init")))
    return st;
  const double res0 = std::sqrt(h2[0]);
  info->initial = res0;
  info->last = res0;
  info->steps = 0;
  info->converged = 0;
  const double tol_eff = std::fmax(ctl->tol, ctl->reduce * res0);
  // a bounded copy wait that ran out inside the first apply voids r0
  if ((st = mfgb_check_device_errors(s))) return st;
  if (res0 <= tol_eff) {
    info->converged = 1;
    return MFGB_OK;
  }
  if (std::isnan(res0)) {
    set_error("mfgb_cg_solve_noalloc: initial residual is NaN");
    return MFGB_ERR_NONFINITE;
  }
  if (ctl->max_steps == 0) return MFGB_ERR_NOT_CONVERGED;

  CgScalars hsc{};
  hsc.rz[0] = h2[1];
  hsc.res[0] = res0;
  hsc.its[0] = 0;
  hsc.tol_eff = tol_eff;
  hsc.max_steps = ctl->max_steps;
  hsc.done = 0;
  if ((st = cuda_status(cudaMemcpyAsync(sc, &hsc, sizeof(hsc), cudaMemcpyHostToDevice, s),
                        "cg scalars")) ||
      (st = cuda_status(cudaMemsetAsync(v, 0, sizeof(double) * n, s), "v = 0")))
    return st;

  const int K = 16;  // iterations between host checks of the done flag
  CgScalars out{};
  for (;;) {
    for (int k = 0; k < K; ++k) {
      const int parity = k & 1;
      if ((st = noalloc_apply(op, v, p, ctl->arith, nullptr, nullptr, s, &sc->done, range_slot,
                              /*accumulate=*/true)))
        return st;
      if (op->n_constrained)
        cg_constrained_copy_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(op->n_constrained,
                                                                      op->d_constrained, p, v, sc);
      cg_dot_pv_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, p, v, pap_part, sc);
      cg_update_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, d_x, r, p, v, dinv, pap_part,
                                                          VEC_BLOCKS, vec_part, sc, parity);
      cg_direction_kernel<<<VEC_BLOCKS, VEC_THREADS, 0, s>>>(n, r, p, v, dinv, vec_part,
                                                             VEC_BLOCKS, sc, parity);
    }
    if ((st = cuda_status(cudaGetLastError(), "cg iterations")) ||
        (st = cuda_status(cudaMemcpyAsync(&out, sc, sizeof(out), cudaMemcpyDeviceToHost, s),
                          "cg scalars copy")) ||
        (st = cuda_status(cudaStreamSynchronize(s), "cg iterations")))
      return st;
    if (out.done) break;
  }
  info->steps = out.final_its;
  info->last = out.final_res;
  info->converged = out.done == 1;
  // reads and clears the device error word (a 4-byte copy, no allocation): a
  // bounded copy wait that ran out in any operator launch of the solve voids x
  if ((st = mfgb_check_device_errors(s))) return st;
  if (out.done == 1) return MFGB_OK;
  if (std::isnan(out.final_res)) {
    set_error("mfgb_cg_solve_noalloc: residual became NaN");
    return MFGB_ERR_NONFINITE;
  }
  set_error("mfgb_cg_solve_noalloc: max_steps reached");
  return MFGB_ERR_NOT_CONVERGED;
}
