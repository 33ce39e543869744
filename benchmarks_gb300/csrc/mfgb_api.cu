// mfgb_api.cu -- C ABI: operator set-up, vmult, kernel seams, diagonal, RHS.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"

namespace mfgb {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

mfgb_status cuda_status(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return MFGB_OK;
  cudaGetLastError();  // clear sticky-free errors
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? MFGB_ERR_OUT_OF_MEMORY : MFGB_ERR_CUDA;
}

// Test hook (mfgb_test_fail_allocation): the n-th device allocation from the
// call on fails as if the device were out of memory; 0 = off.
static std::atomic<int> g_alloc_countdown{0};

bool alloc_hook_fails(const char *what) {
  if (g_alloc_countdown.load() <= 0 || g_alloc_countdown.fetch_sub(1) != 1) return false;
  set_error(std::string(what) + ": allocation failed (injected by mfgb_test_fail_allocation)");
  return true;
}

static mfgb_status dev_alloc(void **p, size_t bytes, const char *what) {
  *p = nullptr;
  if (bytes == 0) return MFGB_OK;
  if (alloc_hook_fails(what)) return MFGB_ERR_OUT_OF_MEMORY;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && bytes > free_b) {
    set_error(std::string(what) + ": needs " + std::to_string(bytes) + " bytes, " +
              std::to_string(free_b) + " free on the device");
    return MFGB_ERR_OUT_OF_MEMORY;
  }
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e, what);
  }
  return MFGB_OK;
}

mfgb_status ensure_df(mfgb_operator *op) {
  if (op->d_Gdf) return MFGB_OK;
  const int64_t nq = op->nq > 0 ? op->nq : op->n;  // G points per direction
  const int64_t ng = op->n_cells * 6 * nq * nq * nq;
  // the pairs carry FP64 accuracy only inside the range window (checked per cell)
  mfgb_status st = range_check_sync(0, nullptr, op->n_cells, (int)(6 * nq * nq * nq), op->d_G,
                                    nullptr, "double-float operator");
  if (!st && op->d_JxW)
    st = range_check_sync(0, nullptr, op->n_cells, op->n * op->n * op->n, op->d_JxW, nullptr,
                          "double-float operator (mass term)");
  if (st) return st;
  // all or nothing: a failed step frees what this call allocated
  auto undo = [&](mfgb_status e) {
    cudaFree(op->d_Gdf);
    cudaFree(op->d_JxWdf);
    op->d_Gdf = nullptr;
    op->d_JxWdf = nullptr;
    return e;
  };
  st = dev_alloc((void **)&op->d_Gdf, sizeof(float2) * ng, "G (double-float)");
  if (st) return undo(st);
  st = cuda_status(g_to_df(ng, op->d_G, op->d_Gdf, nullptr), "G -> double-float");
  if (st) return undo(st);
  if (op->d_JxW) {
    const int64_t nw = op->n_cells * (int64_t)op->n * op->n * op->n;
    if ((st = dev_alloc((void **)&op->d_JxWdf, sizeof(float2) * nw, "JxW (double-float)")) ||
        (st = cuda_status(g_to_df(nw, op->d_JxW, op->d_JxWdf, nullptr), "JxW -> double-float")))
      return undo(st);
  }
  if ((st = cuda_status(cudaDeviceSynchronize(), "G -> double-float"))) return undo(st);
  return MFGB_OK;
}

mfgb_status ensure_fx(mfgb_operator *op) {
  if (op->d_Gfx) return MFGB_OK;
  const int64_t nq = op->nq > 0 ? op->nq : op->n;  // G points per direction
  const int64_t n3 = nq * nq * nq;
  mfgb_status st;
  if ((st = dev_alloc((void **)&op->d_Gfx, sizeof(float2) * op->n_cells * 6 * n3,
                      "G (scaled double-float)")) ||
      (st = dev_alloc((void **)&op->d_Gexp, sizeof(int) * std::max<int64_t>(1, op->n_cells),
                      "G exponent offsets")) ||
      // the mass term's JxW shares the cell's offset with G
      (op->d_JxW && (st = dev_alloc((void **)&op->d_JxWfx, sizeof(float2) * op->n_cells * n3,
                                    "JxW (scaled double-float)"))) ||
      (st = cuda_status(g_to_fx(op->n_cells, (int)(6 * n3), op->d_G, op->d_Gfx, op->d_Gexp, nullptr,
                                op->d_JxW ? (int)n3 : 0, op->d_JxW, op->d_JxWfx),
                        "G -> scaled double-float")) ||
      (st = cuda_status(cudaDeviceSynchronize(), "G -> scaled double-float"))) {
    // all or nothing: the arrays exist only complete
    cudaFree(op->d_Gfx);
    cudaFree(op->d_Gexp);
    cudaFree(op->d_JxWfx);
    op->d_Gfx = nullptr;
    op->d_Gexp = nullptr;
    op->d_JxWfx = nullptr;
    return st;
  }
  return MFGB_OK;
}

mfgb_status ensure_arith(mfgb_operator *op, int arith) {
  if (arith != MFGB_ARITH_FP64_DF || op->n_cells == 0) return MFGB_OK;
  // operators assembled from pairs only (the batched union operators) keep them
  if (!op->d_G) {
    if (op->d_Gdf || op->d_Gfx) return MFGB_OK;
    set_error("operator has no geometric factors");
    return MFGB_ERR_INVALID_ARG;
  }
  // the scaled pairs for GLL collocation (shapes 5 / 6) and the Gauss-point
  // forms (BP3, the Gauss p+1 Laplacian and its Helmholtz form)
  const bool fx = (op->quadrature == 0 && kernel_shape(1, op->n) >= kShapeFx) ||
                  op->quadrature >= 1;
  return fx ? ensure_fx(op) : ensure_df(op);
}

// dst += A src over cells [cell0, cell0 + n) (the map keeps global DoF indices);
// partials/grid (the energy form) are supported by the GLL and Gauss p+1 kernels
static cudaError_t apply_range(mfgb_operator *op, int64_t cell0, int64_t n, double *dst,
                               const double *src, int arith, double *partials, int *grid,
                               cudaStream_t s, const int *done) {
  const int64_t n3 = (int64_t)op->n * op->n * op->n;
  const int64_t q3 = (int64_t)op->nq * op->nq * op->nq;
  const uint32_t *map = op->d_map + cell0 * n3;
  // the Gauss-point forms by the offset-accumulation kernel (no energy partials;
  // the mass term from the JxW pairs built with the G pairs)
  if (op->quadrature >= 1 && arith == MFGB_ARITH_FP64_DF && op->d_Gfx && !partials &&
      (!op->d_JxW || op->d_JxWfx))
    return bp3_fx(op->degree, op->nq, n, map, op->d_Gfx + cell0 * 6 * q3, op->d_Gexp + cell0, src,
                  dst, op->Bq, op->DG, s, done, op->d_JxWfx ? op->d_JxWfx + cell0 * q3 : nullptr);
  if (op->quadrature == 2) {
    if (partials || done) return cudaErrorNotSupported;
    return bp3_apply(op->degree, n, map, op->d_Bq, op->d_DGq, op->Bq, op->DG,
                     op->d_G + cell0 * 6 * q3, op->d_Gdf ? op->d_Gdf + cell0 * 6 * q3 : nullptr,
                     src, dst, arith, s);
  }
  if (arith == MFGB_ARITH_FP64)
    return op->quadrature
               ? bk5g_f64(op->n, n, map, op->d_G + cell0 * 6 * n3, src, dst, op->DG, op->Bq,
                          partials, grid, s, done, op->d_JxW ? op->d_JxW + cell0 * n3 : nullptr)
               : bk5_f64(op->n, n, map, op->d_G + cell0 * 6 * n3, src, dst, op->D, partials, grid,
                         s, done);
  if (op->quadrature)
    return bk5g_df(op->n, n, map, op->d_Gdf + cell0 * 6 * n3, src, dst, op->DG, op->Bq, partials,
                   grid, s, done, op->d_JxWdf ? op->d_JxWdf + cell0 * n3 : nullptr);
  // GLL collocation: the offset-accumulation kernel (no energy partials)
  if (op->d_Gfx && !partials && (kernel_shape(1, op->n) >= kShapeFx || !op->d_Gdf))
    return bk5_fx(op->n, n, map, op->d_Gfx + cell0 * 6 * n3, op->d_Gexp + cell0, src, dst, op->D, s,
                  done);
  return bk5_df(op->n, n, map, op->d_Gdf + cell0 * 6 * n3, src, dst, op->D, partials, grid, s,
                done);
}

mfgb_status vmult_impl(mfgb_operator *op, double *dst, const double *src, int arith,
                       double *partials, int *grid, cudaStream_t s, const int *done) {
  const bool full = partials == nullptr;
  mfgb_status st;
  if (arith != MFGB_ARITH_FP64 && arith != MFGB_ARITH_FP64_DF) {
    set_error("vmult: unknown arith mode");
    return MFGB_ERR_INVALID_ARG;
  }
  if ((st = ensure_arith(op, arith))) return st;
  if (arith == MFGB_ARITH_FP64_DF && !uses_fx(op) && (st = range_check_async(op, op->n_dofs, src, s)))
    return st;
  if (full && (st = cuda_status(cudaMemsetAsync(dst, 0, sizeof(double) * op->n_dofs, s),
                                "vmult: dst = 0")))
    return st;
  if ((st = cuda_status(apply_range(op, 0, op->n_cells, dst, src, arith, partials, grid, s, done),
                        "vmult: operator kernel")))
    return st;
  if (full)
    return cuda_status(copy_constrained(op->n_constrained, op->d_constrained, src, dst, s),
                       "vmult: constrained rows");
  return MFGB_OK;
}

// kernel shape per (arithmetic class, N): 0 column, 1 point-per-thread,
// 2 column with TMA-prefetched geometric factors, 3 / 4 the column / TMA
// kernels at the alternative cells per CTA (AltElems).  Defaults are the fastest
// shape per degree measured on a GB300 at ~3e7 DoFs (autotune.py re-measures).
static int g_shape[3][10] = {
    {0, 0, 4, 3, 2, 4, 2, 1, 2, 1},  // FP64
    {2, 2, 6, 6, 6, 5, 6, 6, 5, 5},  // double-float (5, 6: offset accumulation)
    {0, 0, 3, 3, 0, 3, 2, 4, 4, 2},  // FP32
};

// device-side error word, one per device: bit 0 a TMA wait that ran out of
// time, bit 1 a double-float source vector outside its range
static __device__ int g_device_error;
static int *g_device_error_ptr[64] = {nullptr};
static std::mutex g_device_error_mutex;

// device address of the error word on the current device, looked up once per
// device and cached for the life of the process (a cudaDeviceReset or a
// teardown of the primary context invalidates it)
int *device_error_flag() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_device_error_mutex);
  if (!g_device_error_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_device_error) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    g_device_error_ptr[dev] = (int *)p;
  }
  return g_device_error_ptr[dev];
}

// ---- input range of the double-float kernels without per-cell scaling --------
// A pair keeps 48 significant bits while both of its floats stay normal; with
// the largest magnitude of a vector (per cell for geometric factors) in
// [2^-40, 2^55], results, products and their error terms keep clear of float
// under- and overflow through the operator's sums.
constexpr int kRangeLo = 1023 - 40, kRangeHi = 1023 + 55;  // biased exponents

__device__ __forceinline__ int finite_exp(double x) {
  const int e = (int)(((unsigned)(__double_as_longlong(x) >> 32) >> 20) & 0x7FFu);
  return e == 0x7FF ? 0 : e;
}

__device__ __forceinline__ int block_max(int v, int *s_red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? s_red[threadIdx.x] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  }
  return v;  // valid in thread 0
}

// largest biased exponent of the finite entries of v -> atomicMax(*slot)
__global__ void __launch_bounds__(256) vec_exp_max_kernel(int64_t n, const double *__restrict__ v,
                                                          int *slot) {
  __shared__ int s_red[8];
  int em = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    em = max(em, finite_exp(v[t]));
  em = block_max(em, s_red);
  if (threadIdx.x == 0 && em) atomicMax(slot, em);
}

// *flag |= bit when the (nonzero) largest exponent lies outside the window
__global__ void exp_window_kernel(const int *slot, int *flag, int bit) {
  const int em = *slot;
  if (em && (em < kRangeLo || em > kRangeHi)) atomicOr(flag, bit);
}

// one warp per cell: *flag |= bit when a cell's largest exponent (nonzero cells)
// lies outside the window
__global__ void cell_exp_window_kernel(int64_t n_cells, int per_cell, const double *__restrict__ G,
                                       int *flag, int bit) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = warp; c < n_cells; c += n_warps) {
    int em = 0;
    for (int t = lane; t < per_cell; t += 32) em = max(em, finite_exp(G[c * per_cell + t]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) em = max(em, __shfl_xor_sync(0xFFFFFFFFu, em, o));
    if (lane == 0 && em && (em < kRangeLo || em > kRangeHi)) atomicOr(flag, bit);
  }
}

static unsigned range_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8));
}

// stream-ordered check of a vector (slot: one device int of scratch): the
// device error word gets kDevErrRange when its largest magnitude is outside
// the window
mfgb_status vec_range_check(int *slot, int64_t n, const double *v, cudaStream_t s) {
  int *flag = device_error_flag();
  if (!flag) {
    set_error("range check: no device error word");
    return MFGB_ERR_CUDA;
  }
  if (n <= 0) return MFGB_OK;
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(slot, 0, sizeof(int), s), "range slot = 0"))) return st;
  vec_exp_max_kernel<<<range_grid(n), 256, 0, s>>>(n, v, slot);
  exp_window_kernel<<<1, 1, 0, s>>>(slot, flag, kDevErrRange);
  return cuda_status(cudaGetLastError(), "range check");
}

// the same for per-cell geometric factors
mfgb_status cells_range_check(int64_t n_cells, int per_cell, const double *G, cudaStream_t s) {
  int *flag = device_error_flag();
  if (!flag) {
    set_error("range check: no device error word");
    return MFGB_ERR_CUDA;
  }
  if (n_cells <= 0) return MFGB_OK;
  cell_exp_window_kernel<<<range_grid(n_cells * 32), 256, 0, s>>>(n_cells, per_cell, G, flag,
                                                                    kDevErrRange);
  return cuda_status(cudaGetLastError(), "range check");
}

mfgb_status range_check_async(mfgb_operator *op, int64_t n, const double *v, cudaStream_t s) {
  mfgb_status st;
  if (!op->d_range && (st = dev_alloc((void **)&op->d_range, sizeof(int), "range slot")))
    return st;
  return vec_range_check(op->d_range, n, v, s);
}

// synchronous check of caller arrays (a vector and per-cell geometric
// factors, either may be empty): MFGB_ERR_RANGE when one is outside the window
mfgb_status range_check_sync(int64_t n, const double *v, int64_t n_cells, int per_cell,
                             const double *G, cudaStream_t s, const char *what) {
  int *d = nullptr;
  mfgb_status st;
  if ((st = cuda_status(cudaMallocAsync((void **)&d, 2 * sizeof(int), s), "range scratch")))
    return st;
  int h = 0;
  cudaError_t e = cudaMemsetAsync(d, 0, 2 * sizeof(int), s);
  if (e == cudaSuccess && n > 0) {
    vec_exp_max_kernel<<<range_grid(n), 256, 0, s>>>(n, v, d);
    exp_window_kernel<<<1, 1, 0, s>>>(d, d + 1, 1);
  }
  if (e == cudaSuccess && n_cells > 0)
    cell_exp_window_kernel<<<range_grid(n_cells * 32), 256, 0, s>>>(n_cells, per_cell, G, d + 1,
                                                                      2);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d + 1, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if ((st = cuda_status(e, "range check"))) return st;
  if (h) {
    set_error(std::string(what) + ": " + ((h & 2) ? "geometric factors of a cell" : "an input vector") +
              " with largest magnitude outside [2^-40, 2^55], the range of the double-float "
              "arithmetic without per-cell scaling (use MFGB_ARITH_FP64)");
    return MFGB_ERR_RANGE;
  }
  return MFGB_OK;
}

bool uses_fx(const mfgb_operator *op) {
  if (op->quadrature >= 1) return op->d_Gfx != nullptr && (!op->d_JxW || op->d_JxWfx);
  return op->quadrature == 0 && op->d_Gfx && (kernel_shape(1, op->n) >= kShapeFx || !op->d_Gdf);
}

int kernel_shape(int arith_class, int N) {
  if (arith_class < 0 || arith_class > 2 || N < 0 || N > 9) return 0;
  return g_shape[arith_class][N];
}

mfgb_status apply_add_impl(mfgb_operator *op, double *dst, const double *src, int arith,
                           cudaStream_t s, const int *done) {
  mfgb_status st;
  if (arith != MFGB_ARITH_FP64 && arith != MFGB_ARITH_FP64_DF) {
    set_error("apply: unknown arith mode");
    return MFGB_ERR_INVALID_ARG;
  }
  if ((st = ensure_arith(op, arith))) return st;
  if (arith == MFGB_ARITH_FP64_DF && !uses_fx(op) && (st = range_check_async(op, op->n_dofs, src, s)))
    return st;
  if (done && op->quadrature == 2) done = nullptr;  // the BP3 kernel runs every time
  return cuda_status(apply_range(op, 0, op->n_cells, dst, src, arith, nullptr, nullptr, s, done),
                     "apply: operator kernel");
}

static void free_operator(mfgb_operator *op) {
  if (!op) return;
  cudaFree(op->d_map);
  cudaFree(op->d_G);
  cudaFree(op->d_Gdf);
  cudaFree(op->d_G32);
  cudaFree(op->d_Gfx);
  cudaFree(op->d_Gexp);
  cudaFree(op->d_range);
  cudaFree(op->d_constrained);
  cudaFree(op->d_partials);
  cudaFree(op->d_JxW);
  cudaFree(op->d_JxWdf);
  cudaFree(op->d_JxWfx);
  cudaFree(op->d_hsrc);
  cudaFree(op->d_hdst);
  cudaFree(op->d_Bq);
  cudaFree(op->d_DGq);
  for (cudaStream_t st : op->pipe)
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t e : op->pipe_ev) cudaEventDestroy(e);
  delete op;
}

static void init_basis(mfgb_operator *op, int degree) {
  op->degree = degree;
  op->n = degree + 1;
  op->nq = op->n;
  gll_nodes(op->n, op->gll_x, op->gll_w);
  derivative_matrix(op->n, op->gll_x, op->D);
}

}  // namespace mfgb

using namespace mfgb;

extern "C" {

const char *mfgb_status_string(mfgb_status s) {
  switch (s) {
    case MFGB_OK: return "ok";
    case MFGB_ERR_INVALID_ARG: return "invalid argument";
    case MFGB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case MFGB_ERR_NOT_CONVERGED: return "not converged";
    case MFGB_ERR_TIMEOUT: return "timeout";
    case MFGB_ERR_NONFINITE: return "non-finite value";
    case MFGB_ERR_CUDA: return "CUDA error";
    case MFGB_ERR_UNSUPPORTED: return "unsupported";
    case MFGB_ERR_RANGE: return "input outside the double-float range";
    default: return "unknown status";
  }
}

const char *mfgb_last_error(void) { return g_last_error.c_str(); }

int mfgb_version(void) { return 1; }

mfgb_status mfgb_set_kernel_shape(int arith, int degree, int shape) {
  if (arith < 0 || arith > 2 || degree < 1 || degree > 8 || shape < 0 ||
      shape > (arith == MFGB_ARITH_FP64_DF ? 6 : 4)) {
    set_error("mfgb_set_kernel_shape: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  g_shape[arith][degree + 1] = shape;
  return MFGB_OK;
}

mfgb_status mfgb_test_fail_allocation(int n) {
  if (n < 0) {
    set_error("mfgb_test_fail_allocation: n must be >= 0");
    return MFGB_ERR_INVALID_ARG;
  }
  g_alloc_countdown.store(n);
  return MFGB_OK;
}

mfgb_status mfgb_check_device_errors(void *stream) {
  int *flag = device_error_flag();
  if (!flag) {
    set_error("mfgb_check_device_errors: no device error word");
    return MFGB_ERR_CUDA;
  }
  int h = 0;
  cudaStream_t s = (cudaStream_t)stream;
  mfgb_status st;
  if ((st = cuda_status(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, s),
                        "read device error word")) ||
      (st = cuda_status(cudaMemsetAsync(flag, 0, sizeof(int), s), "clear device error word")) ||
      (st = cuda_status(cudaStreamSynchronize(s), "device error word")))
    return st;
  if (h & kDevErrTimeout) {
    set_error("a kernel's bulk-copy wait exceeded its time limit; results are invalid");
    return MFGB_ERR_TIMEOUT;
  }
  if (h & kDevErrRange) {
    set_error("a double-float operator application got a source vector whose largest magnitude "
              "lies outside [2^-40, 2^55]; its result is invalid (use MFGB_ARITH_FP64)");
    return MFGB_ERR_RANGE;
  }
  return MFGB_OK;
}

mfgb_status mfgb_get_kernel_shape(int arith, int degree, int *shape) {
  if (arith < 0 || arith > 2 || degree < 1 || degree > 8 || !shape) {
    set_error("mfgb_get_kernel_shape: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *shape = g_shape[arith][degree + 1];
  return MFGB_OK;
}

static mfgb_status create_box_impl(const mfgb_box_desc *box, int quadrature, mfgb_operator **out,
                                   const BoxStride *bs = nullptr, bool mass = false);

mfgb_status mfgb_operator_create_box(const mfgb_box_desc *box, mfgb_operator **out) {
  return create_box_impl(box, 0, out);
}

mfgb_status mfgb_operator_create_box_gauss(const mfgb_box_desc *box, mfgb_operator **out) {
  return create_box_impl(box, 1, out);
}

mfgb_status mfgb_operator_create_box_helmholtz(const mfgb_box_desc *box, mfgb_operator **out) {
  return create_box_impl(box, 1, out, nullptr, true);
}

mfgb_status mfgb_operator_create_box_bp3(const mfgb_box_desc *box, mfgb_operator **out) {
  return create_box_impl(box, 2, out);
}

static mfgb_status create_box_impl(const mfgb_box_desc *box, int quadrature, mfgb_operator **out,
                                   const BoxStride *bs, bool mass) {
  if (!box || !out) {
    set_error("mfgb_operator_create_box: null argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (box->degree < 1 || box->degree > 8 || box->nx < 1 || box->ny < 1 || box->nz < 1 ||
      box->geometry_degree < 0 || box->geometry_degree > 8 ||
      !(box->hi[0] > box->lo[0]) || !(box->hi[1] > box->lo[1]) || !(box->hi[2] > box->lo[2])) {
    set_error("mfgb_operator_create_box: degree must be 1..8 and the box non-empty");
    return MFGB_ERR_INVALID_ARG;
  }
  const int64_t p = box->degree;
  const int64_t Nx = p * box->nx + 1, Ny = p * box->ny + 1, Nz = p * box->nz + 1;
  const int64_t n_dofs = Nx * Ny * Nz;
  if (n_dofs >= (int64_t)MFGB_INVALID_DOF) {
    set_error("mfgb_operator_create_box: more DoFs than a 32-bit map can index");
    return MFGB_ERR_UNSUPPORTED;
  }
  mfgb_operator *op = new mfgb_operator();
  init_basis(op, box->degree);
  op->quadrature = quadrature;
  if (quadrature) {  // Gauss points: n (BP5 variant, q = p + 1) or n + 1 (BP3, q = p + 2)
    op->nq = quadrature == 2 ? op->n + 1 : op->n;
    double xq[10], wq[10];
    gauss_nodes(op->nq, xq, wq);
    derivative_matrix(op->nq, xq, op->DG);
    for (int q = 0; q < op->nq; ++q)
      for (int i = 0; i < op->n; ++i) op->Bq[q * op->n + i] = lagrange_value(op->n, op->gll_x, i, xq[q]);
  }
  op->is_box = true;
  op->box = *box;
  op->n_dofs = n_dofs;
  op->n_cells = (int64_t)box->nx * box->ny * box->nz;
  const int64_t n3 = (int64_t)op->n * op->n * op->n;
  const int64_t q3 = (int64_t)op->nq * op->nq * op->nq;  // points per cell of G
  // constrained list: every boundary DoF, ascending
  std::vector<int64_t> cons;
  cons.reserve(2 * (Nx * Ny + Ny * Nz + Nx * Nz));
  for (int64_t gz = 0; gz < Nz; ++gz)
    for (int64_t gy = 0; gy < Ny; ++gy) {
      const bool face = gz == 0 || gz == Nz - 1 || gy == 0 || gy == Ny - 1;
      if (face) {
        for (int64_t gx = 0; gx < Nx; ++gx) cons.push_back(gx + Nx * (gy + Ny * gz));
      } else {
        cons.push_back(Nx * (gy + Ny * gz));
        if (Nx > 1) cons.push_back(Nx - 1 + Nx * (gy + Ny * gz));
      }
    }
  op->n_constrained = (int64_t)cons.size();
  op->h_constrained = cons;
  mfgb_status st;
  if ((st = dev_alloc((void **)&op->d_map, sizeof(uint32_t) * op->n_cells * n3, "dof map")) ||
      (st = dev_alloc((void **)&op->d_G, sizeof(double) * op->n_cells * 6 * q3, "G")) ||
      (st = dev_alloc((void **)&op->d_constrained, sizeof(int64_t) * cons.size(), "constraints")) ||
      (mass && (st = dev_alloc((void **)&op->d_JxW, sizeof(double) * op->n_cells * n3, "JxW"))) ||
      (quadrature == 2 &&
       ((st = dev_alloc((void **)&op->d_Bq, sizeof(double) * op->nq * op->n, "BP3 basis")) ||
        (st = dev_alloc((void **)&op->d_DGq, sizeof(double) * op->nq * op->nq, "BP3 derivative"))))) {
    free_operator(op);
    return st;
  }
  if ((st = cuda_status(cudaMemcpy(op->d_constrained, cons.data(), sizeof(int64_t) * cons.size(),
                                   cudaMemcpyHostToDevice),
                        "constraints copy")) ||
      (st = cuda_status(box_map(*box, op->d_map, nullptr), "box map")) ||
      (st = cuda_status(box_geometry(*box, op->gll_x, op->gll_w, op->D, op->d_G, nullptr,
                                     quadrature != 0, bs, op->d_JxW, op->nq),
                        "box geometry")) ||
      (quadrature == 2 &&
       ((st = cuda_status(cudaMemcpy(op->d_Bq, op->Bq, sizeof(double) * op->nq * op->n,
                                     cudaMemcpyHostToDevice), "BP3 basis")) ||
        (st = cuda_status(cudaMemcpy(op->d_DGq, op->DG, sizeof(double) * op->nq * op->nq,
                                     cudaMemcpyHostToDevice), "BP3 derivative")))) ||
      (st = cuda_status(cudaDeviceSynchronize(), "box set-up"))) {
    free_operator(op);
    return st;
  }
  *out = op;
  return MFGB_OK;
}

mfgb_status mfgb_operator_create(int degree, int64_t n_dofs, int64_t n_cells,
                                 const uint32_t *h_dof_map, const double *h_G,
                                 int64_t n_constrained, const int64_t *h_constrained,
                                 mfgb_operator **out) {
  if (!out || degree < 1 || degree > 8 || n_dofs < 0 || n_cells < 0 || n_constrained < 0 ||
      (n_cells > 0 && (!h_dof_map || !h_G)) || (n_constrained > 0 && !h_constrained) ||
      n_dofs >= (int64_t)MFGB_INVALID_DOF) {
    set_error("mfgb_operator_create: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  *out = nullptr;
  const int64_t n3 = (int64_t)(degree + 1) * (degree + 1) * (degree + 1);
  for (int64_t t = 0; t < n_cells * n3; ++t)
    if (h_dof_map[t] != MFGB_INVALID_DOF && (int64_t)h_dof_map[t] >= n_dofs) {
      set_error("mfgb_operator_create: dof map entry out of range");
      return MFGB_ERR_INVALID_ARG;
    }
  for (int64_t c = 0; c < n_constrained; ++c)
    if (h_constrained[c] < 0 || h_constrained[c] >= n_dofs) {
      set_error("mfgb_operator_create: constrained index out of range");
      return MFGB_ERR_INVALID_ARG;
    }
  mfgb_operator *op = new mfgb_operator();
  init_basis(op, degree);
  op->n_dofs = n_dofs;
  op->n_cells = n_cells;
  op->n_constrained = n_constrained;
  mfgb_status st;
  if ((st = dev_alloc((void **)&op->d_map, sizeof(uint32_t) * n_cells * n3, "dof map")) ||
      (st = dev_alloc((void **)&op->d_G, sizeof(double) * n_cells * 6 * n3, "G")) ||
      (st = dev_alloc((void **)&op->d_constrained, sizeof(int64_t) * n_constrained,
                      "constraints"))) {
    free_operator(op);
    return st;
  }
  if ((n_cells > 0 &&
       ((st = cuda_status(cudaMemcpy(op->d_map, h_dof_map, sizeof(uint32_t) * n_cells * n3,
                                     cudaMemcpyHostToDevice),
                          "map copy")) ||
        (st = cuda_status(cudaMemcpy(op->d_G, h_G, sizeof(double) * n_cells * 6 * n3,
                                     cudaMemcpyHostToDevice),
                          "G copy")))) ||
      (n_constrained > 0 &&
       (st = cuda_status(cudaMemcpy(op->d_constrained, h_constrained,
                                    sizeof(int64_t) * n_constrained, cudaMemcpyHostToDevice),
                         "constraints copy")))) {
    free_operator(op);
    return st;
  }
  *out = op;
  return MFGB_OK;
}

mfgb_status mfgb_operator_destroy(mfgb_operator *op) {
  free_operator(op);
  return MFGB_OK;
}

mfgb_status mfgb_operator_info(const mfgb_operator *op, int64_t *n_dofs, int64_t *n_cells,
                               int *degree, int64_t *n_constrained) {
  if (!op) {
    set_error("mfgb_operator_info: null operator");
    return MFGB_ERR_INVALID_ARG;
  }
  if (n_dofs) *n_dofs = op->n_dofs;
  if (n_cells) *n_cells = op->n_cells;
  if (degree) *degree = op->degree;
  if (n_constrained) *n_constrained = op->n_constrained;
  return MFGB_OK;
}

mfgb_status mfgb_operator_export(const mfgb_operator *op, uint32_t *h_dof_map, double *h_G,
                                 int64_t *h_constrained) {
  if (!op) {
    set_error("mfgb_operator_export: null operator");
    return MFGB_ERR_INVALID_ARG;
  }
  const int64_t n3 = (int64_t)op->n * op->n * op->n;
  const int64_t q3 = (int64_t)op->nq * op->nq * op->nq;  // G points per cell
  mfgb_status st;
  if (h_dof_map && op->n_cells > 0 &&
      (st = cuda_status(cudaMemcpy(h_dof_map, op->d_map, sizeof(uint32_t) * op->n_cells * n3,
                                   cudaMemcpyDeviceToHost),
                        "export map")))
    return st;
  if (h_G && op->n_cells > 0 &&
      (st = cuda_status(cudaMemcpy(h_G, op->d_G, sizeof(double) * op->n_cells * 6 * q3,
                                   cudaMemcpyDeviceToHost),
                        "export G")))
    return st;
  if (h_constrained && op->n_constrained > 0 &&
      (st = cuda_status(cudaMemcpy(h_constrained, op->d_constrained,
                                   sizeof(int64_t) * op->n_constrained, cudaMemcpyDeviceToHost),
                        "export constraints")))
    return st;
  return MFGB_OK;
}

mfgb_status mfgb_vmult(const mfgb_operator *op, double *d_dst, const double *d_src, int arith,
                       void *stream) {
  if (!op || (op->n_dofs > 0 && (!d_dst || !d_src)) || d_dst == d_src) {
    set_error("mfgb_vmult: invalid argument (dst and src must be distinct device vectors)");
    return MFGB_ERR_INVALID_ARG;
  }
  return vmult_impl(const_cast<mfgb_operator *>(op), d_dst, d_src, arith, nullptr, nullptr,
                    (cudaStream_t)stream);
}

mfgb_status mfgb_vmult_add(const mfgb_operator *op, double *d_dst, const double *d_src, int arith,
                           void *stream) {
  if (!op || (op->n_dofs > 0 && (!d_dst || !d_src)) || d_dst == d_src) {
    set_error("mfgb_vmult_add: invalid argument (dst and src must be distinct device vectors)");
    return MFGB_ERR_INVALID_ARG;
  }
  return apply_add_impl(const_cast<mfgb_operator *>(op), d_dst, d_src, arith, (cudaStream_t)stream,
                        nullptr);
}

mfgb_status mfgb_copy_constrained(const mfgb_operator *op, double *d_dst, const double *d_src,
                                  void *stream) {
  if (!op || (op->n_constrained > 0 && (!d_dst || !d_src))) {
    set_error("mfgb_copy_constrained: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  return cuda_status(copy_constrained(op->n_constrained, op->d_constrained, d_src, d_dst,
                                      (cudaStream_t)stream),
                     "mfgb_copy_constrained");
}

static bool read_basis(int degree, const double *d_dbasis, double *D, cudaStream_t s) {
  const int n = degree + 1;
  if (cudaMemcpyAsync(D, d_dbasis, sizeof(double) * n * n, cudaMemcpyDeviceToHost, s) !=
      cudaSuccess)
    return false;
  return cudaStreamSynchronize(s) == cudaSuccess;
}

mfgb_status mfgb_bk5_lvector(int degree, int64_t n_cells, const double *d_dbasis,
                             const double *d_G, const double *d_src, double *d_dst,
                             const uint32_t *d_dof_indices, int arith, void *stream) {
  if (degree < 1 || degree > 8 || n_cells < 0 ||
      (n_cells > 0 && (!d_dbasis || !d_G || !d_src || !d_dst || !d_dof_indices))) {
    set_error("mfgb_bk5_lvector: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (n_cells == 0) return MFGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  double D[81];
  if (!read_basis(degree, d_dbasis, D, s)) return cuda_status(cudaGetLastError(), "read dbasis");
  cudaError_t e;
  if (arith == MFGB_ARITH_FP64)
    e = bk5_f64(degree + 1, n_cells, d_dof_indices, d_G, d_src, d_dst, D, nullptr, nullptr, s);
  else if (arith == MFGB_ARITH_FP64_DF && (reinterpret_cast<uintptr_t>(d_G) & 15u) == 0) {
    // offset double-float with per-cell scaling: any input range, no check
    e = bk5_fx_g64(degree + 1, n_cells, d_dof_indices, d_G, d_src, d_dst, D, s);
  } else if (arith == MFGB_ARITH_FP64_DF) {
    // (the source vector's length is not an argument of this seam: G is checked)
    const int n3 = (degree + 1) * (degree + 1) * (degree + 1);
    mfgb_status st = range_check_sync(0, nullptr, n_cells, 6 * n3, d_G, s, "mfgb_bk5_lvector");
    if (st) return st;
    e = bk5_df_g64(degree + 1, n_cells, d_dof_indices, d_G, d_src, d_dst, D, s);
  }
  else {
    set_error("mfgb_bk5_lvector: unknown arith");
    return MFGB_ERR_INVALID_ARG;
  }
  return cuda_status(e, "mfgb_bk5_lvector");
}

mfgb_status mfgb_bk5_evector(int degree, int64_t nelmt, const double *d_dbasis, const double *d_G,
                             const double *d_in, double *d_out, int arith, void *stream) {
  if (degree < 1 || degree > 8 || nelmt < 0 ||
      (nelmt > 0 && (!d_dbasis || !d_G || !d_in || !d_out))) {
    set_error("mfgb_bk5_evector: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  if (nelmt == 0) return MFGB_OK;
  cudaStream_t s = (cudaStream_t)stream;
  double D[81];
  if (!read_basis(degree, d_dbasis, D, s)) return cuda_status(cudaGetLastError(), "read dbasis");
  cudaError_t e;
  if (arith == MFGB_ARITH_FP64)
    e = bk5_f64(degree + 1, nelmt, nullptr, d_G, d_in, d_out, D, nullptr, nullptr, s);
  else if (arith == MFGB_ARITH_FP64_DF && (reinterpret_cast<uintptr_t>(d_G) & 15u) == 0) {
    // offset double-float with per-element scaling: any input range, no check
    e = bk5_fx_evec(degree + 1, nelmt, d_G, d_in, d_out, D, s);
  } else if (arith == MFGB_ARITH_FP64_DF) {
    const int n3 = (degree + 1) * (degree + 1) * (degree + 1);
    mfgb_status st = range_check_sync(nelmt * n3, d_in, nelmt, 6 * n3, d_G, s, "mfgb_bk5_evector");
    if (st) return st;
    e = bk5_df_g64(degree + 1, nelmt, nullptr, d_G, d_in, d_out, D, s);
  }
  else {
    set_error("mfgb_bk5_evector: unknown arith");
    return MFGB_ERR_INVALID_ARG;
  }
  return cuda_status(e, "mfgb_bk5_evector");
}

static int g_host_slabs = 0;  // slabs of the host-buffer pipeline (0: automatic)

mfgb_status mfgb_set_host_pipeline(int slabs) {
  if (slabs < 0 || slabs > 64) {
    set_error("mfgb_set_host_pipeline: slabs must be 0 (automatic) .. 64");
    return MFGB_ERR_INVALID_ARG;
  }
  g_host_slabs = slabs;
  return MFGB_OK;
}

// vmult on host vectors, pipelined over z-slabs of cells on three streams:
// H2D of the DoF planes a slab adds -> the slab's cells -> D2H of the planes it
// completes (identity rows applied), while the next slab's planes arrive.
// Slab k covers cell layers [z0, z1) and DoF planes p z0 .. p z1; plane p z1 is
// shared with slab k + 1, so it is finished (and copied back) by slab k + 1.
// The copies' ends are moved to page boundaries of the host buffers (below).
mfgb_status mfgb_vmult_host(const mfgb_operator *cop, double *h_dst, const double *h_src, int arith,
                            void *stream) {
  if (!cop || (cop->n_dofs > 0 && (!h_dst || !h_src)) || h_dst == h_src ||
      (arith != MFGB_ARITH_FP64 && arith != MFGB_ARITH_FP64_DF)) {
    set_error("mfgb_vmult_host: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  mfgb_operator *op = const_cast<mfgb_operator *>(cop);
  if (op->n_dofs == 0) return MFGB_OK;
  mfgb_status st;
  if ((st = ensure_arith(op, arith))) return st;
  if (!op->d_hsrc) {
    if ((st = dev_alloc((void **)&op->d_hsrc, sizeof(double) * op->n_dofs, "host apply src")) ||
        (st = dev_alloc((void **)&op->d_hdst, sizeof(double) * op->n_dofs, "host apply dst")))
      return st;
  }
  if (!op->pipe[0])
    for (auto &ps : op->pipe)
      if (cudaStreamCreateWithFlags(&ps, cudaStreamNonBlocking) != cudaSuccess)
        return cuda_status(cudaErrorUnknown, "mfgb_vmult_host: streams");
  const int p = op->degree;
  const int nz = op->is_box ? op->box.nz : 1;
  // >= 2 cell layers a slab; 16 slabs unless set by mfgb_set_host_pipeline
  const int want = g_host_slabs > 0 ? g_host_slabs : 16;
  const int S = op->is_box ? std::max(1, std::min(want, nz / 2)) : 1;
  const int Lz = (nz + S - 1) / S;
  const int n_ev = 3 * S + 1;  // S <= 64
  while ((int)op->pipe_ev.size() < n_ev) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
      return cuda_status(cudaErrorUnknown, "mfgb_vmult_host: events");
    op->pipe_ev.push_back(e);
  }
  cudaStream_t s = (cudaStream_t)stream, s_in = op->pipe[0], s_c = op->pipe[1], s_out = op->pipe[2];
  cudaEvent_t *ev = op->pipe_ev.data();
  // everything after the caller's prior work on its stream
  cudaEventRecord(ev[0], s);
  cudaStreamWaitEvent(s_in, ev[0], 0);
  cudaStreamWaitEvent(s_c, ev[0], 0);
  cudaStreamWaitEvent(s_out, ev[0], 0);
  int64_t plane = op->n_dofs, cells_per_layer = op->n_cells;
  if (op->is_box) {
    plane = ((int64_t)p * op->box.nx + 1) * ((int64_t)p * op->box.ny + 1);
    cells_per_layer = (int64_t)op->box.nx * op->box.ny;
  }
  const int64_t *hc = op->h_constrained.data();
  const int64_t nhc = (int64_t)op->h_constrained.size();
  // Copy boundaries on 4 KiB of host address: copies that start and end inside
  // a page ran about 25 % slower in both directions (4.7 -> 3.8 ms a step at
  // 67.6M DoFs).  H2D ends are rounded up (a slab's cells get all their DoFs
  // early; the extra DoFs carry the same values again), D2H ends down (the rest
  // of the completed DoFs go with the next slab).
  constexpr uintptr_t kPage = 4096;
  auto page_up = [&](const double *base, int64_t i) {
    const uintptr_t adr = reinterpret_cast<uintptr_t>(base + i);
    return std::min(op->n_dofs, i + (int64_t)(((adr + kPage - 1) / kPage * kPage - adr) / 8));
  };
  auto page_down = [&](const double *base, int64_t i) {
    return i - (int64_t)((reinterpret_cast<uintptr_t>(base + i) % kPage) / 8);
  };
  int64_t h2d_done = 0, d2h_done = 0;  // DoFs [0, x) already copied
  int last_out = -1;
  for (int k = 0, z0 = 0; z0 < nz; ++k, z0 += Lz) {
    const int z1 = std::min(nz, z0 + Lz);
    const bool last = z1 == nz;
    // DoFs [a, b) this slab adds; [c0, c1) it completes
    int64_t a, b, c0, c1;
    if (op->is_box) {
      a = (k == 0 ? 0 : ((int64_t)p * z0 + 1)) * plane;
      b = ((int64_t)p * z1 + 1) * plane;
      c0 = (int64_t)p * z0 * plane;
      c1 = last ? op->n_dofs : (int64_t)p * z1 * plane;
    } else {
      a = 0; b = op->n_dofs; c0 = 0; c1 = op->n_dofs;
    }
    const int64_t h_end = last ? op->n_dofs : std::max(h2d_done, page_up(h_src, b));
    if (h_end > h2d_done)
      cudaMemcpyAsync(op->d_hsrc + h2d_done, h_src + h2d_done, sizeof(double) * (h_end - h2d_done),
                      cudaMemcpyHostToDevice, s_in);
    h2d_done = h_end;
    cudaEventRecord(ev[1 + 3 * k], s_in);
    cudaStreamWaitEvent(s_c, ev[1 + 3 * k], 0);
    cudaMemsetAsync(op->d_hdst + a, 0, sizeof(double) * (b - a), s_c);
    const int64_t cell0 = (int64_t)z0 * cells_per_layer, ncell = (int64_t)(z1 - z0) * cells_per_layer;
    if ((st = cuda_status(apply_range(op, op->is_box ? cell0 : 0, op->is_box ? ncell : op->n_cells,
                                      op->d_hdst, op->d_hsrc, arith, nullptr, nullptr, s_c,
                                      nullptr),
                          "mfgb_vmult_host: kernel")))
      return st;
    // identity rows among the completed DoFs (the list is ascending)
    const int64_t i0 = op->is_box ? std::lower_bound(hc, hc + nhc, c0) - hc : 0;
    const int64_t i1 = op->is_box ? std::lower_bound(hc, hc + nhc, c1) - hc : op->n_constrained;
    if (i1 > i0 &&
        (st = cuda_status(copy_constrained(i1 - i0, op->d_constrained + i0, op->d_hsrc, op->d_hdst,
                                           s_c),
                          "mfgb_vmult_host: constrained rows")))
      return st;
    cudaEventRecord(ev[2 + 3 * k], s_c);
    cudaStreamWaitEvent(s_out, ev[2 + 3 * k], 0);
    const int64_t d_end = last ? op->n_dofs : std::max(d2h_done, page_down(h_dst, c1));
    if (d_end > d2h_done)
      cudaMemcpyAsync(h_dst + d2h_done, op->d_hdst + d2h_done, sizeof(double) * (d_end - d2h_done),
                      cudaMemcpyDeviceToHost, s_out);
    d2h_done = d_end;
    cudaEventRecord(ev[3 + 3 * k], s_out);
    last_out = 3 + 3 * k;
  }
  cudaStreamWaitEvent(s, ev[last_out], 0);
  // double-float kernels without per-cell scaling: the uploaded source's range
  if (arith == MFGB_ARITH_FP64_DF && !uses_fx(op) &&
      (st = range_check_async(op, op->n_dofs, op->d_hsrc, s)))
    return st;
  return cuda_status(cudaGetLastError(), "mfgb_vmult_host");
}

mfgb_status mfgb_compute_diagonal(const mfgb_operator *op, double *d_diag, void *stream) {
  if (!op || (op->n_dofs > 0 && !d_diag)) {
    set_error("mfgb_compute_diagonal: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  mfgb_status st;
  if ((st = cuda_status(cudaMemsetAsync(d_diag, 0, sizeof(double) * op->n_dofs, s), "diag = 0")))
    return st;
  if (op->quadrature)
    st = cuda_status(diagonal_gauss(op->n, op->nq, op->n_cells, op->d_map, op->d_G, op->d_JxW,
                                    op->Bq, op->DG, d_diag, s),
                     "diagonal kernel (Gauss points)");
  else
    st = cuda_status(diagonal_f64(op->n, op->n_cells, op->d_map, op->d_G, op->D, d_diag, s),
                     "diagonal kernel");
  if (st) return st;
  return cuda_status(set_constrained(op->n_constrained, op->d_constrained, d_diag, 1.0, s),
                     "diagonal constrained rows");
}

mfgb_status mfgb_invert_diagonal(int64_t n, double *d_diag, void *stream) {
  if (n < 0 || (n > 0 && !d_diag)) {
    set_error("mfgb_invert_diagonal: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  return cuda_status(invert_diagonal(n, d_diag, (cudaStream_t)stream), "invert diagonal");
}

mfgb_status mfgb_rhs_uniform(const mfgb_operator *op, uint64_t seed, double *d_b, void *stream) {
  if (!op || (op->n_dofs > 0 && !d_b)) {
    set_error("mfgb_rhs_uniform: invalid argument");
    return MFGB_ERR_INVALID_ARG;
  }
  std::vector<double> b(op->n_dofs);
  std::mt19937_64 gen(seed);
  for (int64_t i = 0; i < op->n_dofs; ++i)
    b[i] = 2.0 * ((double)(gen() >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
  cudaStream_t s = (cudaStream_t)stream;
  mfgb_status st;
  if ((st = cuda_status(cudaMemcpyAsync(d_b, b.data(), sizeof(double) * op->n_dofs,
                                        cudaMemcpyHostToDevice, s),
                        "rhs copy")) ||
      (st = cuda_status(set_constrained(op->n_constrained, op->d_constrained, d_b, 0.0, s),
                        "rhs constrained")))
    return st;
  return cuda_status(cudaStreamSynchronize(s), "rhs sync");
}

}  // extern "C"

mfgb_status mfgb::create_box_strided(const mfgb_box_desc *box, const BoxStride *bs,
                                     mfgb_operator **out) {
  return create_box_impl(box, 0, out, bs);
}
