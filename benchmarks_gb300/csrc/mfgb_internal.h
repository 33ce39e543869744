// mfgb_internal.h -- host-side internals shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>

#include <vector>

#include "mfgb.h"

struct mfgb_operator {
  int degree = 0;
  int n = 0;  // points per direction
  int64_t n_dofs = 0, n_cells = 0, n_constrained = 0;
  uint32_t *d_map = nullptr;      // [n_cells][n^3]
  double *d_G = nullptr;          // [n_cells][6][n^3]
  float2 *d_Gdf = nullptr;        // same, double-float pairs (built on demand)
  float *d_G32 = nullptr;         // same, FP32 (built on demand)
  float2 *d_Gfx = nullptr;        // GLL operators: G * 2^-gexp[cell] as float pairs (built on demand)
  int *d_Gexp = nullptr;          // the per-cell exponent offsets of d_Gfx
  int *d_range = nullptr;         // slot of the double-float input range check
  int64_t *d_constrained = nullptr;
  double D[81] = {0};             // derivative matrix D[q*n + b]
  double gll_x[9] = {0}, gll_w[9] = {0};
  int quadrature = 0;             // 0: GLL collocation, 1: Gauss p+1 (BP5 variant), 2: Gauss p+2 (BP3)
  int nq = 0;                     // quadrature points per direction (n, or n + 1 for BP3)
  double *d_Bq = nullptr, *d_DGq = nullptr;  // BP3: the two matrices below on the device
  double *d_JxW = nullptr;        // Gauss form with a mass term (Helmholtz): [n_cells][n^3]
  float2 *d_JxWdf = nullptr;      // same, double-float pairs
  float2 *d_JxWfx = nullptr;      // same, times 2^-gexp[cell] of d_Gfx as float pairs
  double DG[100] = {0};           // Gauss forms: collocation derivative on the Gauss points
  double Bq[100] = {0};           // Gauss forms: GLL basis at the Gauss points, Bq[q*n + i]
  bool is_box = false;
  mfgb_box_desc box{};
  // workspace for reductions (per-CTA partials)
  double *d_partials = nullptr;
  int partials_cap = 0;
  // host-buffer apply (mfgb_vmult_host): device copies of the vectors, the
  // constrained rows on the host (ascending), streams and events of the pipeline
  double *d_hsrc = nullptr, *d_hdst = nullptr;
  std::vector<int64_t> h_constrained;
  cudaStream_t pipe[3] = {nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> pipe_ev;
};

namespace mfgb {

void set_error(const std::string &msg);
// true when the allocation test hook makes this device allocation fail (every
// device allocation of the library asks first; mfgb_api.cu)
bool alloc_hook_fails(const char *what);
mfgb_status cuda_status(cudaError_t e, const char *what);

// 1D bases (host, FP64)
void gll_nodes(int n, double *x, double *w);
double lagrange_derivative(int n, const double *nodes, int j, double x);
double lagrange_value(int n, const double *nodes, int j, double x);
void derivative_matrix(int n, const double *nodes, double *D);

// BK5 kernels (map == nullptr selects E-vector mode where supported)
cudaError_t bk5_f64(int N, int64_t n_cells, const uint32_t *map, const double *G, const double *src,
                    double *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                    const int *done = nullptr);
cudaError_t bk5_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const double *src,
                   double *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                    const int *done = nullptr);
// FP64-accurate collocation operator with offset double-float accumulation and
// per-cell scaling (mfgb_bk5_fx.cu); G = the scaled pairs, gexp their offsets
cudaError_t bk5_fx(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                   const double *src, double *dst, const double *D, cudaStream_t s,
                   const int *done = nullptr);
// the BK6 vector Laplacian on the scaled pairs of bk5_fx: src / dst hold 3
// interleaved components per DoF, each component scaled per cell on its own
cudaError_t bk6_fx(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const int *gexp,
                   const double *src, double *dst, const double *D, cudaStream_t s);
// bk5_fx on the caller's FP64 G[cell][6][N^3] (16-byte aligned) scaled per
// cell inside the kernel, for the BK5 L-vector seam: dst += A src through map
cudaError_t bk5_fx_g64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                       const double *src, double *dst, const double *D, cudaStream_t s);
// the E-vector form of bk5_fx for the BK5 E-vector seam: the caller's FP64
// G[e][6][N^3] (16-byte aligned) scaled per element inside the kernel,
// contiguous src / dst (dst overwritten)
cudaError_t bk5_fx_evec(int N, int64_t nelmt, const double *G, const double *src, double *dst,
                        const double *D, cudaStream_t s);
// per-cell scaled float pairs of G (and of JxW, with the same per-cell offset)
cudaError_t g_to_fx(int64_t n_cells, int per_cell, const double *G, float2 *Gfx, int *gexp,
                    cudaStream_t s, int per_cell_j = 0, const double *J = nullptr,
                    float2 *Jfx = nullptr);
cudaError_t bk5_df_g64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                       const double *src, double *dst, const double *D, cudaStream_t s,
                       const int *done = nullptr);
cudaError_t bk5_f32(int N, int64_t n_cells, const uint32_t *map, const float *G, const float *src,
                    float *dst, const double *D, double *partials, int *grid, cudaStream_t s,
                    const int *done = nullptr);

// Gauss-quadrature form (mfgb_bk5g.cu)
// (jxw != nullptr adds the mass term: the Helmholtz form)
cudaError_t bk5g_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                     const double *src, double *dst, const double *DG, const double *B,
                     double *partials, int *grid, cudaStream_t s, const int *done = nullptr,
                     const double *jxw = nullptr);
cudaError_t bk5g_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G,
                    const double *src, double *dst, const double *DG, const double *B,
                    double *partials, int *grid, cudaStream_t s, const int *done = nullptr,
                    const float2 *jxw = nullptr);
void gauss_nodes(int n, double *x, double *w);

// assembled diagonal with per-cell weights: d_i = sum_e w_e (A_e)_ii (mfgb_mlp.cu)
cudaError_t weighted_diagonal(const mfgb_operator *op, const double *w, double *diag,
                              cudaStream_t s);

// BK6 vector Laplacian, 3 interleaved components (mfgb_bk6.cu)
cudaError_t bk6_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                    const double *src, double *dst, const double *D, cudaStream_t s);
cudaError_t bk6_df(int N, int64_t n_cells, const uint32_t *map, const float2 *G, const double *src,
                   double *dst, const double *D, cudaStream_t s);

// set-up kernels (mfgb_setup.cu)
cudaError_t box_map(const mfgb_box_desc &b, uint32_t *d_map, cudaStream_t s);
// A coarsened box level: cell c of an axis spans fine mesh nodes
// [min(c s, nf), min((c+1) s, nf)] of a uniform nf-cell axis, so the levels
// of any nf stay nested (only the last cell of an axis can be narrower).
// b.nx = ceil(nf[0] / s) etc.; s <= 1 is the uniform box itself.
struct BoxStride {
  int nf[3];
  int s;
};
cudaError_t box_geometry(const mfgb_box_desc &b, const double *gll_x, const double *gll_w,
                         const double *D, double *d_G, cudaStream_t s, bool at_gauss = false,
                         const BoxStride *bs = nullptr, double *d_JxW = nullptr,
                         int n_gauss = 0);  // Gauss points per direction (0: degree + 1)
// exact diagonal of the Gauss-point operator (Laplacian, plus mass when JxW is
// given) on a box, accumulated into diag (not zeroed; constrained rows untouched)
cudaError_t diagonal_gauss(int N, int NQ, int64_t n_cells, const uint32_t *map, const double *G,
                           const double *JxW, const double *B, const double *DG, double *diag,
                           cudaStream_t s);
// device-side dot product (mfgb_cg.cu): *out = a.b, stream ordered, without a
// host synchronisation; partials holds dot_partials_count() doubles
int dot_partials_count();
cudaError_t dot_to_device(int64_t n, const double *a, const double *b, double *partials,
                          double *out, cudaStream_t s);

// BP3 operator (nq = degree + 2) and Gauss p+1 Laplacian (nq = degree + 1)
// with offset double-float accumulation (mfgb_bp3_fx.cu): dst += A src over
// n_cells cells, scaled G pairs Gfx[cell][6][nq^3] with per-cell exponent
// offsets gexp, host copies of the basis hB[q*nm+i] and the Gauss-point
// derivative hDG[q*nq+m]; done (may be null): skip when *done is set; jxw
// (may be null): the mass term's JxW[cell][nq^3] pairs on the scale of Gfx
cudaError_t bp3_fx(int degree, int nq, int64_t n_cells, const uint32_t *map, const float2 *Gfx,
                   const int *gexp, const double *src, double *dst, const double *hB,
                   const double *hDG, cudaStream_t s, const int *done,
                   const float2 *jxw = nullptr);
// the Helmholtz form of bp3_fx (nq = degree + 1, mfgb_helmholtz_fx.cu): the
// Gauss p+1 Laplacian plus the mass term from jxw, JxW pairs [cell][nq^3] on
// the scale of Gfx
cudaError_t helmholtz_fx(int degree, int64_t n_cells, const uint32_t *map, const float2 *Gfx,
                         const int *gexp, const float2 *jxw, const double *src, double *dst,
                         const double *hB, const double *hDG, cudaStream_t s, const int *done);
// CEED BK1 mass operator on E-vectors with offset double-float accumulation and
// per-element scaling (mfgb_bp3_fx.cu): out = B^T (JxW o B in) per element,
// host copy of the basis hB[q*nm+i], nq = degree + 2
cudaError_t bk1_fx(int degree, int64_t nelmt, const double *in, const double *JxW, double *out,
                   const double *hB, cudaStream_t s);
// CEED BK3 Laplacian on E-vectors with offset double-float accumulation and
// per-element scaling of the input and of the caller's FP64 G[e][6][nq^3]
// (16-byte aligned; mfgb_bp3_fx.cu), nq = degree + 2
cudaError_t bk3_fx(int degree, int64_t nelmt, const double *G, const double *in, double *out,
                   const double *hB, const double *hDG, cudaStream_t s);
// BK1 E-vector mass operator on the FP64 tensor cores (mfgb_bk1_dmma.cu),
// degree 1..6, the layouts of mfgb_bk1_evector
cudaError_t bk1_dmma(int degree, int64_t nelmt, const double *basis, const double *JxW,
                     const double *in, double *out, cudaStream_t s);
// BP3 operator (mfgb_bkq.cu): dst += A src, q = p + 2 Gauss points, G[cell][6][nq^3]
// in FP64 (G) and, for double-float arithmetic, as pairs (Gdf); the bases on the
// device (d_B, d_DG) and on the host (h_B, h_DG)
cudaError_t bp3_apply(int degree, int64_t n_cells, const uint32_t *map, const double *d_B,
                      const double *d_DG, const double *h_B, const double *h_DG, const double *G,
                      const float2 *Gdf, const double *src, double *dst, int arith,
                      cudaStream_t s);
cudaError_t g_to_df(int64_t n, const double *G, float2 *Gdf, cudaStream_t s);
cudaError_t g_to_f32(int64_t n, const double *G, float *G32, cudaStream_t s);
cudaError_t diagonal_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                         const double *D, double *diag, cudaStream_t s);
cudaError_t set_constrained(int64_t n_constrained, const int64_t *constrained, double *v,
                            double value, cudaStream_t s);
cudaError_t copy_constrained(int64_t n_constrained, const int64_t *constrained, const double *src,
                             double *dst, cudaStream_t s);
cudaError_t invert_diagonal(int64_t n, double *d, cudaStream_t s);

// operator helpers (mfgb_api.cu)
mfgb_status create_box_strided(const mfgb_box_desc *box, const BoxStride *bs,
                               mfgb_operator **out);
// kernel shape table (arithmetic class 0 FP64, 1 double-float, 2 FP32; N = p + 1);
// double-float shapes >= kShapeFx select the offset-accumulation kernel
int kernel_shape(int arith_class, int N);
constexpr int kShapeFx = 5;
// bits of the device error word (mfgb_check_device_errors)
constexpr int kDevErrTimeout = 1, kDevErrRange = 2;
// the double-float input range (mfgb_api.cu): stream-ordered check of a source
// vector into the device error word, and a synchronous check of caller arrays
mfgb_status range_check_async(mfgb_operator *op, int64_t n, const double *v, cudaStream_t s);
mfgb_status vec_range_check(int *slot, int64_t n, const double *v, cudaStream_t s);
mfgb_status cells_range_check(int64_t n_cells, int per_cell, const double *G, cudaStream_t s);
mfgb_status range_check_sync(int64_t n, const double *v, int64_t n_cells, int per_cell,
                             const double *G, cudaStream_t s, const char *what);
// true when double-float applies of op run the per-cell scaled kernel
bool uses_fx(const mfgb_operator *op);
mfgb_status ensure_df(mfgb_operator *op);
// the copy of G the FP64_DF arithmetic of apply_range reads: the scaled pairs of
// the offset-accumulation kernel for GLL operators, the plain pairs otherwise
mfgb_status ensure_fx(mfgb_operator *op);
mfgb_status ensure_arith(mfgb_operator *op, int arith);
mfgb_status ensure_partials(mfgb_operator *op, int n);
// dst += A src (cell loop only: no zeroing, no identity rows); `done` lets
// a captured solver iteration skip the work once converged
mfgb_status apply_add_impl(mfgb_operator *op, double *dst, const double *src, int arith,
                           cudaStream_t s, const int *done);
// vmult with optional energy partials (p.Ap) for the solver
mfgb_status vmult_impl(mfgb_operator *op, double *dst, const double *src, int arith,
                       double *partials, int *grid, cudaStream_t s, const int *done = nullptr);

}  // namespace mfgb
