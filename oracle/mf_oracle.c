/*
 * mf_oracle.c -- CPU ORACLE (test infrastructure only) for the BK5/BP5
 * matrix-free Laplacian.  See mf_oracle.h for conventions.  Only tests/,
 * the smoke check and bench.py's CPU-baseline leg load this code.
 *
 * Reference files followed (paths relative to dealii-X/benchmarks):
 *   sum_factorization/include/math/lagrange_basis.hpp:9-70     Lagrange basis
 *   CEED_BK/include/kernels/BK5/templated_cuda_kernels.cuh:50-122 BK5 E-vector
 *   bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:129-151  gather + mask
 *   bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:406-426  atomic scatter
 *   bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:123-167
 *       vmult: dst = 0, cell loop, copy_constrained_values
 *   bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:229-292
 *       G = JxW * Jinv Jinv^T (index order as in the deal.II-kernel variant
 *       portable_laplace_operator.h:227-255: grad_phys = Jinv^T grad_ref)
 *   bp5_kokkos/benchmark.cc:218-251  diagonal + inverse with the d<=0 guard
 *   bp5_kokkos/benchmark.cc:355-378, scaling_bp35_kokkos_kernel/program.cc:
 *       263-287  SolverCG + ReductionControl (deal.II, third party, >= 9.7.0;
 *       the published conjugate-gradient algorithm is restated here)
 */
#include "mf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* 1D bases                                                                  */
/* ------------------------------------------------------------------------ */

/* Legendre P_{N-1}(x) and P_N(x) by the three-term recurrence. */
static void legendre_pair(int N, double x, double *pm1, double *pN) {
  double p0 = 1.0, p1 = x;
  if (N == 0) { *pm1 = 0.0; *pN = 1.0; return; }
  for (int k = 2; k <= N; ++k) {
    double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  *pm1 = p0;
  *pN = p1;
}

/* Gauss-Lobatto-Legendre nodes/weights on [-1,1], ascending.  Newton's
   method on x P_N(x) - P_{N-1}(x) (whose interior zeros are those of P_N'),
   started at the Chebyshev-Gauss-Lobatto points; w = 2 / (N (N+1) P_N^2).
   (Published method: Canuto et al., "Spectral Methods", sec. 2.3; the
   iteration as in G. von Winckel's lglnodes.)  Symmetrised afterwards. */
void orc_gll(int n, double *x, double *w) {
  if (n == 1) { x[0] = 0.0; w[0] = 2.0; return; }
  const int N = n - 1;
  for (int i = 0; i < n; ++i) {
    double xi = -cos(M_PI * i / N);
    for (int it = 0; it < 200; ++it) {
      double pm1, pN;
      legendre_pair(N, xi, &pm1, &pN);
      double dx = (xi * pN - pm1) / ((N + 1.0) * pN);
      xi -= dx;
      if (fabs(dx) < 1e-17) break;
    }
    double pm1, pN;
    legendre_pair(N, xi, &pm1, &pN);
    x[i] = xi;
    w[i] = 2.0 / (N * (N + 1.0) * pN * pN);
  }
  for (int i = 0; i < n / 2; ++i) {
    double v = 0.5 * (x[N - i] - x[i]);
    double ww = 0.5 * (w[N - i] + w[i]);
    x[i] = -v; x[N - i] = v;
    w[i] = ww; w[N - i] = ww;
  }
  if (n % 2) x[n / 2] = 0.0;
  x[0] = -1.0; x[N] = 1.0;
}

/* Gauss-Legendre nodes/weights on [-1,1], ascending (Newton on P_n). */
void orc_gauss(int n, double *x, double *w) {
  for (int i = 0; i < n; ++i) {
    double xi = -cos(M_PI * (i + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 200; ++it) {
      double pm1, pn;
      legendre_pair(n, xi, &pm1, &pn);
      dp = n * (xi * pn - pm1) / (xi * xi - 1.0);
      double dx = pn / dp;
      xi -= dx;
      if (fabs(dx) < 1e-17) break;
    }
    double pm1, pn;
    legendre_pair(n, xi, &pm1, &pn);
    dp = n * (xi * pn - pm1) / (xi * xi - 1.0);
    x[i] = xi;
    w[i] = 2.0 / ((1.0 - xi * xi) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) {
    double v = 0.5 * (x[n - 1 - i] - x[i]);
    double ww = 0.5 * (w[n - 1 - i] + w[i]);
    x[i] = -v; x[n - 1 - i] = v;
    w[i] = ww; w[n - 1 - i] = ww;
  }
  if (n % 2) x[n / 2] = 0.0;
}

/* l_j(x) = prod_{m != j} (x - x_m) / prod_{m != j} (x_j - x_m)
   (sum_factorization/include/math/lagrange_basis.hpp:10-42) */
double orc_lagrange_value(int n, const double *nodes, int j, double x) {
  double num = 1.0, den = 1.0;
  for (int m = 0; m < n; ++m) {
    if (m == j) continue;
    num *= (x - nodes[m]);
    den *= (nodes[j] - nodes[m]);
  }
  return num / den;
}

/* l_j'(x) = sum_{i != j} 1/(x_j - x_i) prod_{m != i,j} (x - x_m)/(x_j - x_m)
   (sum_factorization/include/math/lagrange_basis.hpp:44-65) */
double orc_lagrange_derivative(int n, const double *nodes, int j, double x) {
  double sum = 0.0;
  for (int i = 0; i < n; ++i) {
    if (i == j) continue;
    double prod = 1.0;
    for (int m = 0; m < n; ++m)
      if (m != i && m != j) prod *= (x - nodes[m]) / (nodes[j] - nodes[m]);
    sum += (1.0 / (nodes[j] - nodes[i])) * prod;
  }
  return sum;
}

/* D[point*n + basis] = l_basis'(x_point)  (CEED_BK dbasis layout,
   CEED_BK/include/kernels/BK5/templated_cuda_kernels.cuh:55-58,85-86) */
void orc_derivative_matrix(int n, const double *nodes, double *D) {
  for (int q = 0; q < n; ++q)
    for (int b = 0; b < n; ++b) D[q * n + b] = orc_lagrange_derivative(n, nodes, b, nodes[q]);
}

/* B[t*n_from + f] = l_f(pts_to[t]) */
void orc_interpolation_matrix(int n_from, const double *nodes_from, int n_to,
                              const double *pts_to, double *B) {
  for (int t = 0; t < n_to; ++t)
    for (int f = 0; f < n_from; ++f)
      B[t * n_from + f] = orc_lagrange_value(n_from, nodes_from, f, pts_to[t]);
}

/* ------------------------------------------------------------------------ */
/* structured box mesh                                                       */
/* ------------------------------------------------------------------------ */

int64_t orc_box_n_dofs(const orc_box *b) {
  const int64_t p = b->degree;
  return (p * b->nx + 1) * (p * b->ny + 1) * (p * b->nz + 1);
}

int64_t orc_box_n_cells(const orc_box *b) {
  return (int64_t)b->nx * b->ny * b->nz;
}

static int geo_degree(const orc_box *b) {
  return b->geometry_degree > 0 ? b->geometry_degree : b->degree;
}

void orc_box_cell_nodes(const orc_box *b, int64_t cell, double *xyz) {
  const int n = geo_degree(b) + 1;
  double xg[16], wg[16];
  orc_gll(n, xg, wg);
  const int64_t c[3] = {cell % b->nx, (cell / b->nx) % b->ny, cell / ((int64_t)b->nx * b->ny)};
  const int strided = b->stride > 1;
  const int s = strided ? b->stride : 1;
  const int nc[3] = {b->nx, b->ny, b->nz};
  double h[3], a[3], w[3];  /* node range [a, a + w) of the cell in units of h */
  for (int d = 0; d < 3; ++d) {
    const int64_t nf = strided ? b->nf[d] : nc[d];
    const int64_t lo = c[d] * s < nf ? c[d] * s : nf, hi = (c[d] + 1) * s < nf ? (c[d] + 1) * s : nf;
    h[d] = (b->hi[d] - b->lo[d]) / (double)nf;
    a[d] = (double)lo;
    w[d] = (double)(hi - lo);
  }
  const double two_pi = 2.0 * M_PI;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        const double X = b->lo[0] + (a[0] + 0.5 * (xg[k] + 1.0) * w[0]) * h[0];
        const double Y = b->lo[1] + (a[1] + 0.5 * (xg[j] + 1.0) * w[1]) * h[1];
        const double Z = b->lo[2] + (a[2] + 0.5 * (xg[i] + 1.0) * w[2]) * h[2];
        const double s = b->amplitude * sin(two_pi * X) * sin(two_pi * Y) * sin(two_pi * Z);
        double *o = xyz + 3 * (i * n * n + j * n + k);
        o[0] = X + s;
        o[1] = Y + s;
        o[2] = Z + s;
      }
}

int64_t orc_box_dof_map(const orc_box *b, uint32_t *map, int64_t *constrained) {
  const int p = b->degree, n = p + 1;
  const int64_t Nx = (int64_t)p * b->nx + 1, Ny = (int64_t)p * b->ny + 1, Nz = (int64_t)p * b->nz + 1;
  const int64_t n_cells = orc_box_n_cells(b);
  if (map) {
    for (int64_t e = 0; e < n_cells; ++e) {
      const int64_t cx = e % b->nx, cy = (e / b->nx) % b->ny, cz = e / ((int64_t)b->nx * b->ny);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
          for (int k = 0; k < n; ++k) {
            const int64_t gx = cx * p + k, gy = cy * p + j, gz = cz * p + i;
            const int bnd = gx == 0 || gx == Nx - 1 || gy == 0 || gy == Ny - 1 || gz == 0 || gz == Nz - 1;
            map[e * n * n * n + i * n * n + j * n + k] =
                bnd ? ORC_INVALID_DOF : (uint32_t)(gx + Nx * (gy + Ny * gz));
          }
    }
  }
  int64_t nc = 0;
  for (int64_t gz = 0; gz < Nz; ++gz)
    for (int64_t gy = 0; gy < Ny; ++gy)
      for (int64_t gx = 0; gx < Nx; ++gx) {
        const int bnd = gx == 0 || gx == Nx - 1 || gy == 0 || gy == Ny - 1 || gz == 0 || gz == Nz - 1;
        if (bnd) {
          if (constrained) constrained[nc] = gx + Nx * (gy + Ny * gz);
          ++nc;
        }
      }
  return nc;
}

/* G_ab = JxW sum_d Jinv[a][d] Jinv[b][d], J[d][a] = dx_d/dxi_a, JxW = |det J| w.
   Returns 1 if the cell is degenerate or folded (det changes sign / is 0). */
int orc_cell_geometry(int n, const double *D, const double *w, const double *xyz, double *Gc) {
  const int nq = n * n * n;
  int bad = 0, sign0 = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        double J[3][3];
        for (int d = 0; d < 3; ++d) {
          double jr = 0, js = 0, jt = 0;
          for (int m = 0; m < n; ++m) {
            jr += D[i * n + m] * xyz[3 * (m * n * n + j * n + k) + d];
            js += D[j * n + m] * xyz[3 * (i * n * n + m * n + k) + d];
            jt += D[k * n + m] * xyz[3 * (i * n * n + j * n + m) + d];
          }
          J[d][0] = jr; J[d][1] = js; J[d][2] = jt;
        }
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const int sg = det > 0 ? 1 : (det < 0 ? -1 : 0);
        if (sg == 0) bad = 1;
        if (sign0 == 0) sign0 = sg; else if (sg != sign0) bad = 1;
        /* Jinv[a][d] = cofactor(d,a) / det */
        double Ji[3][3];
        Ji[0][0] = c00 / det;
        Ji[1][0] = c01 / det;
        Ji[2][0] = c02 / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        const double jxw = fabs(det) * w[i] * w[j] * w[k];
        const int q = i * n * n + j * n + k;
        int c = 0;
        for (int a = 0; a < 3; ++a)
          for (int bb = a; bb < 3; ++bb) {
            double s = 0;
            for (int d = 0; d < 3; ++d) s += Ji[a][d] * Ji[bb][d];
            Gc[c * nq + q] = jxw * s;
            ++c;
          }
      }
  return bad;
}

/* Same as orc_cell_geometry with the Jacobian of the Q_{ng-1} geometry
   interpolant evaluated at the n GLL points per direction:
   dx/dxi_r (i,j,k) = sum_abc Dv[i][a] V[j][b] V[k][c] x_abc (and cyclic). */
static int cell_geometry_general(int n, int ng, const double *V, const double *Dv, const double *w,
                                 const double *xyz, double *Gc, double *JxWc);

int orc_cell_geometry_general(int n, int ng, const double *V, const double *Dv, const double *w,
                              const double *xyz, double *Gc) {
  return cell_geometry_general(n, ng, V, Dv, w, xyz, Gc, NULL);
}

/* the same, also writing JxW per point when JxWc != NULL */
static int cell_geometry_general(int n, int ng, const double *V, const double *Dv, const double *w,
                                 const double *xyz, double *Gc, double *JxWc) {
  const int nq = n * n * n, ng2 = ng * ng;
  int bad = 0, sign0 = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        double J[3][3] = {{0}};
        for (int a = 0; a < ng; ++a)
          for (int bb = 0; bb < ng; ++bb)
            for (int c = 0; c < ng; ++c) {
              const double *x = xyz + 3 * (a * ng2 + bb * ng + c);
              const double wr = Dv[i * ng + a] * V[j * ng + bb] * V[k * ng + c];
              const double ws = V[i * ng + a] * Dv[j * ng + bb] * V[k * ng + c];
              const double wt = V[i * ng + a] * V[j * ng + bb] * Dv[k * ng + c];
              for (int d = 0; d < 3; ++d) {
                J[d][0] += wr * x[d];
                J[d][1] += ws * x[d];
                J[d][2] += wt * x[d];
              }
            }
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const int sg = det > 0 ? 1 : (det < 0 ? -1 : 0);
        if (sg == 0) bad = 1;
        if (sign0 == 0) sign0 = sg; else if (sg != sign0) bad = 1;
        double Ji[3][3];
        Ji[0][0] = c00 / det;
        Ji[1][0] = c01 / det;
        Ji[2][0] = c02 / det;
        Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        const double jxw = fabs(det) * w[i] * w[j] * w[k];
        const int q = i * n * n + j * n + k;
        if (JxWc) JxWc[q] = jxw;
        if (JxWc) JxWc[q] = jxw;
        int c = 0;
        for (int a = 0; a < 3; ++a)
          for (int bb = a; bb < 3; ++bb) {
            double s = 0;
            for (int d = 0; d < 3; ++d) s += Ji[a][d] * Ji[bb][d];
            Gc[c * nq + q] = jxw * s;
            ++c;
          }
      }
  return bad;
}

int64_t orc_box_geometry(const orc_box *b, double *G) {
  const int n = b->degree + 1, nq = n * n * n;
  const int ng = geo_degree(b) + 1, ngq = ng * ng * ng;
  double xg[16], wg[16], D[256], xgeo[16], wgeo[16], V[256], Dv[256];
  orc_gll(n, xg, wg);
  orc_derivative_matrix(n, xg, D);
  orc_gll(ng, xgeo, wgeo);
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < ng; ++a) {
      V[i * ng + a] = orc_lagrange_value(ng, xgeo, a, xg[i]);
      Dv[i * ng + a] = orc_lagrange_derivative(ng, xgeo, a, xg[i]);
    }
  const int64_t n_cells = orc_box_n_cells(b);
  int64_t bad = 0;
#pragma omp parallel reduction(+ : bad)
  {
    double *xyz = (double *)malloc(sizeof(double) * 3 * ngq);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < n_cells; ++e) {
      orc_box_cell_nodes(b, e, xyz);
      if (ng == n)
        bad += orc_cell_geometry(n, D, wg, xyz, G + e * 6 * nq);
      else
        bad += orc_cell_geometry_general(n, ng, V, Dv, wg, xyz, G + e * 6 * nq);
    }
    free(xyz);
  }
  return bad;
}

/* ------------------------------------------------------------------------ */
/* operator                                                                  */
/* ------------------------------------------------------------------------ */

/* One element: out = D^T G D in  (CEED_BK/include/kernels/BK5/
   templated_cuda_kernels.cuh:50-122, with G[6][n^3] read per component). */
static void bk5_element(int n, const double *D, const double *G, const double *u, double *out,
                        double *vr, double *vs, double *vt) {
  const int nq = n * n * n;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        const int q = i * n * n + j * n + k;
        double qr = 0, qs = 0, qt = 0;
        for (int m = 0; m < n; ++m) {
          qr += D[i * n + m] * u[m * n * n + j * n + k];
          qs += D[j * n + m] * u[i * n * n + m * n + k];
          qt += D[k * n + m] * u[i * n * n + j * n + m];
        }
        const double grr = G[0 * nq + q], grs = G[1 * nq + q], grt = G[2 * nq + q];
        const double gss = G[3 * nq + q], gst = G[4 * nq + q], gtt = G[5 * nq + q];
        vr[q] = grr * qr + grs * qs + grt * qt;
        vs[q] = grs * qr + gss * qs + gst * qt;
        vt[q] = grt * qr + gst * qs + gtt * qt;
      }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) {
        double t = 0;
        for (int m = 0; m < n; ++m) t += D[m * n + i] * vr[m * n * n + j * n + k];
        for (int m = 0; m < n; ++m) t += D[m * n + j] * vs[i * n * n + m * n + k];
        for (int m = 0; m < n; ++m) t += D[m * n + k] * vt[i * n * n + j * n + m];
        out[i * n * n + j * n + k] = t;
      }
}

void orc_bk5_evector(int n, int64_t nelmt, const double *D, const double *G,
                     const double *in, double *out) {
  const int nq = n * n * n;
#pragma omp parallel
  {
    double *scratch = (double *)malloc(sizeof(double) * 3 * nq);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelmt; ++e)
      bk5_element(n, D, G + e * 6 * nq, in + e * nq, out + e * nq, scratch, scratch + nq,
                  scratch + 2 * nq);
    free(scratch);
  }
}

void orc_bk5_apply(int n, int64_t n_cells, const uint32_t *map, const double *D,
                   const double *G, int64_t n_dofs, int64_t n_constrained,
                   const int64_t *constrained, const double *src, double *dst) {
  const int nq = n * n * n;
  memset(dst, 0, sizeof(double) * n_dofs);
#pragma omp parallel
  {
    double *scratch = (double *)malloc(sizeof(double) * 5 * nq);
    double *u = scratch, *y = scratch + nq;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < n_cells; ++e) {
      const uint32_t *me = map + e * nq;
      for (int l = 0; l < nq; ++l) u[l] = me[l] == ORC_INVALID_DOF ? 0.0 : src[me[l]];
      bk5_element(n, D, G + e * 6 * nq, u, y, scratch + 2 * nq, scratch + 3 * nq, scratch + 4 * nq);
      for (int l = 0; l < nq; ++l)
        if (me[l] != ORC_INVALID_DOF) {
#pragma omp atomic
          dst[me[l]] += y[l];
        }
    }
    free(scratch);
  }
  for (int64_t c = 0; c < n_constrained; ++c) dst[constrained[c]] = src[constrained[c]];
}

void orc_bk5_diagonal(int n, int64_t n_cells, const uint32_t *map, const double *D,
                      const double *G, int64_t n_dofs, int64_t n_constrained,
                      const int64_t *constrained, double *diag) {
  const int nq = n * n * n;
  memset(diag, 0, sizeof(double) * n_dofs);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < n_cells; ++e) {
    const uint32_t *me = map + e * nq;
    const double *Ge = G + e * 6 * nq;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
          const int q = i * n * n + j * n + k;
          if (me[q] == ORC_INVALID_DOF) continue;
          double d = 0;
          for (int a = 0; a < n; ++a) d += Ge[0 * nq + a * n * n + j * n + k] * D[a * n + i] * D[a * n + i];
          for (int a = 0; a < n; ++a) d += Ge[3 * nq + i * n * n + a * n + k] * D[a * n + j] * D[a * n + j];
          for (int a = 0; a < n; ++a) d += Ge[5 * nq + i * n * n + j * n + a] * D[a * n + k] * D[a * n + k];
          d += 2.0 * Ge[1 * nq + q] * D[i * n + i] * D[j * n + j];
          d += 2.0 * Ge[2 * nq + q] * D[i * n + i] * D[k * n + k];
          d += 2.0 * Ge[4 * nq + q] * D[j * n + j] * D[k * n + k];
#pragma omp atomic
          diag[me[q]] += d;
        }
  }
  for (int64_t c = 0; c < n_constrained; ++c) diag[constrained[c]] = 1.0;
}

/* bp5_kokkos/benchmark.cc:240-250 */
void orc_invert_diagonal(int64_t n, double *d) {
  for (int64_t i = 0; i < n; ++i) d[i] = d[i] > 0 ? 1.0 / d[i] : 1.0;
}

/* ------------------------------------------------------------------------ */
/* Gauss-quadrature operator (BP5-variant q = p+1, BP3 q = p+2)               */
/* ------------------------------------------------------------------------ */

void orc_gauss_basis_matrices(int p, int nq, double *B, double *DG) {
  const int n = p + 1;
  double xg[16], wg[16], xq[16], wq[16];
  orc_gll(n, xg, wg);
  orc_gauss(nq, xq, wq);
  for (int q = 0; q < nq; ++q)
    for (int i = 0; i < n; ++i) B[q * n + i] = orc_lagrange_value(n, xg, i, xq[q]);
  orc_derivative_matrix(nq, xq, DG);
}

int64_t orc_box_geometry_gauss(const orc_box *b, int nq, double *Gg) {
  return orc_box_geometry_gauss_jxw(b, nq, Gg, NULL);
}

int64_t orc_box_geometry_gauss_jxw(const orc_box *b, int nq, double *Gg, double *JxW) {
  const int ng = geo_degree(b) + 1, ngq = ng * ng * ng, nq3 = nq * nq * nq;
  double xgeo[16], wgeo[16], xq[16], wq[16], V[256], Dv[256];
  orc_gll(ng, xgeo, wgeo);
  orc_gauss(nq, xq, wq);
  for (int i = 0; i < nq; ++i)
    for (int a = 0; a < ng; ++a) {
      V[i * ng + a] = orc_lagrange_value(ng, xgeo, a, xq[i]);
      Dv[i * ng + a] = orc_lagrange_derivative(ng, xgeo, a, xq[i]);
    }
  const int64_t n_cells = orc_box_n_cells(b);
  int64_t bad = 0;
#pragma omp parallel reduction(+ : bad)
  {
    double *xyz = (double *)malloc(sizeof(double) * 3 * ngq);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < n_cells; ++e) {
      orc_box_cell_nodes(b, e, xyz);
      bad += cell_geometry_general(nq, ng, V, Dv, wq, xyz, Gg + e * 6 * nq3,
                                   JxW ? JxW + e * nq3 : NULL);
    }
    free(xyz);
  }
  return bad;
}

/* apply the 1D matrix M (rows x cols, M[r*cols + c]) along one direction of a
   tensor t[a][b][c] with extents (e0, e1, e2); dir 0 contracts a, 2 contracts c;
   transpose uses M^T */
static void contract(const double *M, int rows, int cols, int dir, int transpose, const int *ext,
                     const double *in, double *out) {
  const int e0 = ext[0], e1 = ext[1], e2 = ext[2];
  const int nin = transpose ? rows : cols, nout = transpose ? cols : rows;
  const int o0 = dir == 0 ? nout : e0, o1 = dir == 1 ? nout : e1, o2 = dir == 2 ? nout : e2;
  for (int a = 0; a < o0; ++a)
    for (int bb = 0; bb < o1; ++bb)
      for (int c = 0; c < o2; ++c) {
        double s = 0;
        for (int m = 0; m < nin; ++m) {
          const double w = transpose ? M[m * cols + (dir == 0 ? a : dir == 1 ? bb : c)]
                                     : M[(dir == 0 ? a : dir == 1 ? bb : c) * cols + m];
          const int ia = dir == 0 ? m : a, ib = dir == 1 ? m : bb, ic = dir == 2 ? m : c;
          s += w * in[(ia * e1 + ib) * e2 + ic];
        }
        out[(a * o1 + bb) * o2 + c] = s;
      }
}

/* one cell: y = B^T D_G^T G D_G B u  (u, y: n^3 GLL nodal values) */
static void bk5g_element(int n, int nq, const double *B, const double *DG, const double *G,
                         const double *W, const double *u, double *y, double *w) {
  const int nq3 = nq * nq * nq;
  double *t1 = w, *t2 = w + nq3, *uq = w + 2 * nq3, *vr = w + 3 * nq3, *vs = w + 4 * nq3,
         *vt = w + 5 * nq3, *acc = w + 6 * nq3, *t3 = w + 7 * nq3;
  int e_nnn[3] = {n, n, n}, e_qnn[3] = {nq, n, n}, e_qqn[3] = {nq, nq, n}, e_qqq[3] = {nq, nq, nq};
  /* values at the Gauss points */
  contract(B, nq, n, 0, 0, e_nnn, u, t1);
  contract(B, nq, n, 1, 0, e_qnn, t1, t2);
  contract(B, nq, n, 2, 0, e_qqn, t2, uq);
  /* collocation gradient, metric */
  contract(DG, nq, nq, 0, 0, e_qqq, uq, t1);
  contract(DG, nq, nq, 1, 0, e_qqq, uq, t2);
  contract(DG, nq, nq, 2, 0, e_qqq, uq, t3);
  for (int q = 0; q < nq3; ++q) {
    const double qr = t1[q], qs = t2[q], qt = t3[q];
    const double grr = G[0 * nq3 + q], grs = G[1 * nq3 + q], grt = G[2 * nq3 + q];
    const double gss = G[3 * nq3 + q], gst = G[4 * nq3 + q], gtt = G[5 * nq3 + q];
    vr[q] = grr * qr + grs * qs + grt * qt;
    vs[q] = grs * qr + gss * qs + gst * qt;
    vt[q] = grt * qr + gst * qs + gtt * qt;
  }
  /* transpose gradient */
  contract(DG, nq, nq, 0, 1, e_qqq, vr, acc);
  contract(DG, nq, nq, 1, 1, e_qqq, vs, t1);
  for (int q = 0; q < nq3; ++q) acc[q] += t1[q];
  contract(DG, nq, nq, 2, 1, e_qqq, vt, t1);
  for (int q = 0; q < nq3; ++q) acc[q] += t1[q];
  /* mass term (Helmholtz form, bp5_kokkos/benchmark.cc:93): JxW u at the points */
  if (W)
    for (int q = 0; q < nq3; ++q) acc[q] += W[q] * uq[q];
  /* back to the GLL nodal values */
  int e_qqq2[3] = {nq, nq, nq}, e_qqn2[3] = {nq, nq, n}, e_qnn2[3] = {nq, n, n};
  contract(B, nq, n, 2, 1, e_qqq2, acc, t2);
  contract(B, nq, n, 1, 1, e_qqn2, t2, t1);
  contract(B, nq, n, 0, 1, e_qnn2, t1, y);
}

/* BK3 E-vector (CEED_BK/include/kernels/BK3/serial_kernels.hpp:29-188): per
   element, interpolation to nq points (basis[q*nm + i]), collocation derivative
   there (dbasis[q*nq + m]), metric G[e][6][nq^3] (point index dir 0 slowest, the
   layout of the reference's CUDA BK3 kernel, templated_cuda_kernels.cuh:156-161),
   transposes back to the nm^3 modes.  in/out [e][nm^3]. */
void orc_bk3_evector(int nm, int nq, int64_t nelmt, const double *basis, const double *dbasis,
                     const double *G, const double *in, double *out) {
  const int nm3 = nm * nm * nm, nq3 = nq * nq * nq;
#pragma omp parallel
  {
    double *w = (double *)malloc(sizeof(double) * 8 * nq3);
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelmt; ++e)
      bk5g_element(nm, nq, basis, dbasis, G + e * 6 * nq3, NULL, in + e * nm3, out + e * nm3, w);
    free(w);
  }
}

/* BK1 E-vector mass operator (CEED_BK/include/kernels/BK1/serial_kernels.hpp:20-121):
   out_e = B^T (JxW_e o (B x B x B) in_e), JxW[e][nq^3] with the point index
   dir 0 slowest (the serial kernel's layout, :80-86). */
void orc_bk1_evector(int nm, int nq, int64_t nelmt, const double *basis, const double *JxW,
                     const double *in, double *out) {
  const int nm3 = nm * nm * nm, nq3 = nq * nq * nq;
  int e_mmm[3] = {nm, nm, nm}, e_qmm[3] = {nq, nm, nm}, e_qqm[3] = {nq, nq, nm},
      e_qqq[3] = {nq, nq, nq};
#pragma omp parallel
  {
    double *t1 = (double *)malloc(sizeof(double) * 2 * nq3), *t2 = t1 + nq3;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < nelmt; ++e) {
      contract(basis, nq, nm, 0, 0, e_mmm, in + e * nm3, t1);
      contract(basis, nq, nm, 1, 0, e_qmm, t1, t2);
      contract(basis, nq, nm, 2, 0, e_qqm, t2, t1);
      for (int q = 0; q < nq3; ++q) t1[q] *= JxW[e * nq3 + q];
      contract(basis, nq, nm, 2, 1, e_qqq, t1, t2);
      contract(basis, nq, nm, 1, 1, e_qqm, t2, t1);
      contract(basis, nq, nm, 0, 1, e_qmm, t1, out + e * nm3);
    }
    free(t1);
  }
}

static void bkg_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                      const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                      int64_t n_constrained, const int64_t *constrained, const double *src,
                      double *dst);

void orc_bk5g_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                    const uint32_t *map, const double *Gg, int64_t n_dofs, int64_t n_constrained,
                    const int64_t *constrained, const double *src, double *dst) {
  bkg_apply(n, nq, B, DG, n_cells, map, Gg, NULL, n_dofs, n_constrained, constrained, src, dst);
}

/* Step64::HelmholtzOperator::vmult (bp5_kokkos/benchmark.cc:195-205): mass +
   stiffness at the Gauss points, dst = 0, cell loop, identity rows */
void orc_helmholtz_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                         const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                         int64_t n_constrained, const int64_t *constrained, const double *src,
                         double *dst) {
  bkg_apply(n, nq, B, DG, n_cells, map, Gg, JxW, n_dofs, n_constrained, constrained, src, dst);
}

/* exact diagonal of the Gauss-point operator (plus mass when JxW != NULL), the
   result of MatrixFreeTools::compute_diagonal (bp5_kokkos/benchmark.cc:231-236),
   1 on constrained rows (not inverted) */
void orc_gauss_diagonal(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                        const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                        int64_t n_constrained, const int64_t *constrained, double *diag) {
  const int n3 = n * n * n, nq3 = nq * nq * nq;
  double DB[256];
  for (int q = 0; q < nq; ++q)
    for (int a = 0; a < n; ++a) {
      double d = 0;
      for (int m = 0; m < nq; ++m) d += DG[q * nq + m] * B[m * n + a];
      DB[q * n + a] = d;
    }
  memset(diag, 0, sizeof(double) * n_dofs);
  for (int64_t e = 0; e < n_cells; ++e) {
    const double *G = Gg + e * 6 * nq3;
    for (int l = 0; l < n3; ++l) {
      const uint32_t dof = map[e * n3 + l];
      if (dof == ORC_INVALID_DOF) continue;
      const int a = l / (n * n), bb = (l / n) % n, c = l % n;
      double acc = 0;
      for (int i = 0; i < nq; ++i)
        for (int j = 0; j < nq; ++j)
          for (int k = 0; k < nq; ++k) {
            const int q = (i * nq + j) * nq + k;
            const double r = DB[i * n + a] * B[j * n + bb] * B[k * n + c];
            const double sv = B[i * n + a] * DB[j * n + bb] * B[k * n + c];
            const double t = B[i * n + a] * B[j * n + bb] * DB[k * n + c];
            const double ph = B[i * n + a] * B[j * n + bb] * B[k * n + c];
            acc += G[q] * r * r + G[3 * nq3 + q] * sv * sv + G[5 * nq3 + q] * t * t +
                   2.0 * (G[nq3 + q] * r * sv + G[2 * nq3 + q] * r * t + G[4 * nq3 + q] * sv * t) +
                   (JxW ? JxW[e * nq3 + q] * ph * ph : 0.0);
          }
      diag[dof] += acc;
    }
  }
  for (int64_t i = 0; i < n_constrained; ++i) diag[constrained[i]] = 1.0;
}

static void bkg_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                      const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                      int64_t n_constrained, const int64_t *constrained, const double *src,
                      double *dst) {
  const int n3 = n * n * n, nq3 = nq * nq * nq;
  memset(dst, 0, sizeof(double) * n_dofs);
#pragma omp parallel
  {
    double *u = (double *)malloc(sizeof(double) * (2 * n3 + 8 * nq3));
    double *y = u + n3, *w = u + 2 * n3;
#pragma omp for schedule(static)
    for (int64_t e = 0; e < n_cells; ++e) {
      const uint32_t *me = map + e * n3;
      for (int l = 0; l < n3; ++l) u[l] = me[l] == ORC_INVALID_DOF ? 0.0 : src[me[l]];
      bk5g_element(n, nq, B, DG, Gg + e * 6 * nq3, JxW ? JxW + e * nq3 : NULL, u, y, w);
      for (int l = 0; l < n3; ++l)
        if (me[l] != ORC_INVALID_DOF) {
#pragma omp atomic
          dst[me[l]] += y[l];
        }
    }
    free(u);
  }
  for (int64_t c = 0; c < n_constrained; ++c) dst[constrained[c]] = src[constrained[c]];
}

void orc_box_rhs_unit_gauss(const orc_box *b, int nq, int64_t n_constrained,
                            const int64_t *constrained, double *rhs) {
  const int n = b->degree + 1, n3 = n * n * n, nq3 = nq * nq * nq;
  const int64_t n_cells = orc_box_n_cells(b), N = orc_box_n_dofs(b);
  double *Gg = (double *)malloc(sizeof(double) * 6 * nq3 * n_cells);
  double *jxw = (double *)malloc(sizeof(double) * nq3 * n_cells);
  uint32_t *map = (uint32_t *)malloc(sizeof(uint32_t) * n3 * n_cells);
  /* JxW at the Gauss points: recompute det J from the geometry (Gg holds G) */
  const int ng = geo_degree(b) + 1;
  double xgeo[16], wgeo[16], xq[16], wq[16], V[256], Dv[256], xgl[16], wgl[16], B[256];
  orc_gll(ng, xgeo, wgeo);
  orc_gauss(nq, xq, wq);
  orc_gll(n, xgl, wgl);
  for (int i = 0; i < nq; ++i) {
    for (int a = 0; a < ng; ++a) {
      V[i * ng + a] = orc_lagrange_value(ng, xgeo, a, xq[i]);
      Dv[i * ng + a] = orc_lagrange_derivative(ng, xgeo, a, xq[i]);
    }
    for (int a = 0; a < n; ++a) B[i * n + a] = orc_lagrange_value(n, xgl, a, xq[i]);
  }
  orc_box_dof_map(b, map, NULL);
  memset(rhs, 0, sizeof(double) * N);
  double *xyz = (double *)malloc(sizeof(double) * 3 * ng * ng * ng);
  for (int64_t e = 0; e < n_cells; ++e) {
    orc_box_cell_nodes(b, e, xyz);
    for (int p = 0; p < nq; ++p)
      for (int q = 0; q < nq; ++q)
        for (int r = 0; r < nq; ++r) {
          double J[3][3] = {{0}};
          for (int a = 0; a < ng; ++a)
            for (int bb = 0; bb < ng; ++bb)
              for (int c = 0; c < ng; ++c) {
                const double *x = xyz + 3 * ((a * ng + bb) * ng + c);
                const double wr = Dv[p * ng + a] * V[q * ng + bb] * V[r * ng + c];
                const double ws = V[p * ng + a] * Dv[q * ng + bb] * V[r * ng + c];
                const double wt = V[p * ng + a] * V[q * ng + bb] * Dv[r * ng + c];
                for (int d = 0; d < 3; ++d) {
                  J[d][0] += wr * x[d];
                  J[d][1] += ws * x[d];
                  J[d][2] += wt * x[d];
                }
              }
          const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                             J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                             J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
          jxw[e * nq3 + (p * nq + q) * nq + r] = fabs(det) * wq[p] * wq[q] * wq[r];
        }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
          const uint32_t dof = map[e * n3 + (i * n + j) * n + k];
          if (dof == ORC_INVALID_DOF) continue;
          double s = 0;
          for (int p = 0; p < nq; ++p)
            for (int q = 0; q < nq; ++q)
              for (int r = 0; r < nq; ++r)
                s += B[p * n + i] * B[q * n + j] * B[r * n + k] * jxw[e * nq3 + (p * nq + q) * nq + r];
          rhs[dof] += s;
        }
  }
  for (int64_t c = 0; c < n_constrained; ++c) rhs[constrained[c]] = 0.0;
  free(xyz); free(map); free(jxw); free(Gg);
}

/* ------------------------------------------------------------------------ */
/* MT19937-64 (Matsumoto & Nishimura, 2000/2004 published algorithm)        */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint64_t mt[312];
  int idx;
} mt64;

static void mt64_seed(mt64 *s, uint64_t seed) {
  s->mt[0] = seed;
  for (int i = 1; i < 312; ++i)
    s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
  s->idx = 312;
}

static uint64_t mt64_next(mt64 *s) {
  const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
  if (s->idx >= 312) {
    for (int i = 0; i < 312; ++i) {
      uint64_t x = (s->mt[i] & UM) | (s->mt[(i + 1) % 312] & LM);
      uint64_t xa = x >> 1;
      if (x & 1ULL) xa ^= 0xB5026F5AA96619E9ULL;
      s->mt[i] = s->mt[(i + 156) % 312] ^ xa;
    }
    s->idx = 0;
  }
  uint64_t y = s->mt[s->idx++];
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  y ^= (y >> 43);
  return y;
}

uint64_t orc_mt19937_64_nth(uint64_t seed, int64_t nth) {
  mt64 s;
  mt64_seed(&s, seed);
  uint64_t v = 0;
  for (int64_t i = 0; i < nth; ++i) v = mt64_next(&s);
  return v;
}

/* b_i = 2 * ((x >> 11) * 2^-53) - 1 for every DoF in index order, then 0 on
   the constrained DoFs. */
void orc_rhs_uniform(uint64_t seed, int64_t n_dofs, int64_t n_constrained,
                     const int64_t *constrained, double *b) {
  mt64 s;
  mt64_seed(&s, seed);
  for (int64_t i = 0; i < n_dofs; ++i) {
    const double u = (double)(mt64_next(&s) >> 11) * (1.0 / 9007199254740992.0);
    b[i] = 2.0 * u - 1.0;
  }
  for (int64_t c = 0; c < n_constrained; ++c) b[constrained[c]] = 0.0;
}

/* ------------------------------------------------------------------------ */
/* conjugate gradients (deal.II SolverCG + ReductionControl semantics)       */
/* ------------------------------------------------------------------------ */
static double dot(int64_t n, const double *a, const double *b) {
  double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

orc_solve_info orc_cg_solve_op(orc_apply_fn apply, void *ctx, int64_t N,
                               const double *diag_inv, const double *b, double *x,
                               orc_reduction_control ctl) {
  orc_solve_info info = {0, 0.0, 0.0, 0};
  double *r = (double *)malloc(sizeof(double) * N);
  double *z = (double *)malloc(sizeof(double) * N);
  double *p = (double *)malloc(sizeof(double) * N);
  double *v = (double *)malloc(sizeof(double) * N);

  /* r = b - A x */
  apply(ctx, x, v);
  for (int64_t i = 0; i < N; ++i) r[i] = b[i] - v[i];
  double res = sqrt(dot(N, r, r));
  info.initial = res;
  info.last = res;
  /* ReductionControl::check at step 0: tol_eff = max(tol, reduce * r0) */
  const double tol_eff = fmax(ctl.tol, ctl.reduce * res);
  if (res <= tol_eff) { info.converged = 1; goto done; }
  if (isnan(res)) goto done;

  for (int64_t i = 0; i < N; ++i) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
  memcpy(p, z, sizeof(double) * N);
  double rz = dot(N, r, z);

  for (int it = 1;; ++it) {
    apply(ctx, p, v);
    const double alpha = rz / dot(N, p, v);
    for (int64_t i = 0; i < N; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * v[i];
    }
    res = sqrt(dot(N, r, r));
    info.steps = it;
    info.last = res;
    if (res <= tol_eff) { info.converged = 1; break; }
    if (it >= ctl.max_steps || isnan(res)) break;
    for (int64_t i = 0; i < N; ++i) z[i] = diag_inv ? diag_inv[i] * r[i] : r[i];
    const double rz_new = dot(N, r, z);
    const double beta = rz_new / rz;
    rz = rz_new;
    for (int64_t i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
  }
done:
  free(r); free(z); free(p); free(v);
  return info;
}

typedef struct {
  int n;
  int64_t n_cells, N, nc;
  const uint32_t *map;
  const double *D, *G;
  const int64_t *c;
} gll_ctx;

static void gll_apply(void *vc, const double *src, double *dst) {
  gll_ctx *c = (gll_ctx *)vc;
  orc_bk5_apply(c->n, c->n_cells, c->map, c->D, c->G, c->N, c->nc, c->c, src, dst);
}

orc_solve_info orc_cg_solve(int n, int64_t n_cells, const uint32_t *map, const double *D,
                            const double *G, int64_t N, int64_t n_constrained,
                            const int64_t *constrained, const double *diag_inv,
                            const double *b, double *x, orc_reduction_control ctl) {
  gll_ctx c = {n, n_cells, N, n_constrained, map, D, G, constrained};
  return orc_cg_solve_op(gll_apply, &c, N, diag_inv, b, x, ctl);
}

typedef struct {
  int n, nq;
  const double *B, *DG;
  int64_t n_cells, N, nc;
  const uint32_t *map;
  const double *G;
  const int64_t *c;
} gauss_ctx;

static void gauss_apply(void *vc, const double *src, double *dst) {
  gauss_ctx *c = (gauss_ctx *)vc;
  orc_bk5g_apply(c->n, c->nq, c->B, c->DG, c->n_cells, c->map, c->G, c->N, c->nc, c->c, src, dst);
}

typedef struct {
  gauss_ctx g;
  const double *JxW;
} helmholtz_ctx;

static void helmholtz_apply_cb(void *vc, const double *src, double *dst) {
  helmholtz_ctx *h = (helmholtz_ctx *)vc;
  gauss_ctx *c = &h->g;
  orc_helmholtz_apply(c->n, c->nq, c->B, c->DG, c->n_cells, c->map, c->G, h->JxW, c->N, c->nc,
                      c->c, src, dst);
}

orc_solve_info orc_cg_solve_helmholtz(int n, int nq, const double *B, const double *DG,
                                      int64_t n_cells, const uint32_t *map, const double *Gg,
                                      const double *JxW, int64_t N, int64_t n_constrained,
                                      const int64_t *constrained, const double *diag_inv,
                                      const double *b, double *x, orc_reduction_control ctl) {
  helmholtz_ctx h = {{n, nq, B, DG, n_cells, N, n_constrained, map, Gg, constrained}, JxW};
  return orc_cg_solve_op(helmholtz_apply_cb, &h, N, diag_inv, b, x, ctl);
}

orc_solve_info orc_cg_solve_gauss(int n, int nq, const double *B, const double *DG,
                                  int64_t n_cells, const uint32_t *map, const double *Gg,
                                  int64_t N, int64_t n_constrained, const int64_t *constrained,
                                  const double *diag_inv, const double *b, double *x,
                                  orc_reduction_control ctl) {
  gauss_ctx c = {n, nq, B, DG, n_cells, N, n_constrained, map, Gg, constrained};
  return orc_cg_solve_op(gauss_apply, &c, N, diag_inv, b, x, ctl);
}
