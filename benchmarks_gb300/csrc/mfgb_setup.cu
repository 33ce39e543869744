// mfgb_setup.cu -- bases, structured-box set-up kernels, diagonal, constraints.
#include <algorithm>
#include <cmath>

#include "mfgb_common.cuh"
#include "mfgb_internal.h"

namespace mfgb {

// ------------------------------------------------------------------ bases --
static void legendre_pair(int N, double x, double *pm1, double *pN) {
  double p0 = 1.0, p1 = x;
  if (N == 0) { *pm1 = 0.0; *pN = 1.0; return; }
  for (int k = 2; k <= N; ++k) {
    const double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
    p0 = p1;
    p1 = pk;
  }
  *pm1 = p0;
  *pN = p1;
}

// Gauss-Lobatto-Legendre points: Newton on x P_N - P_{N-1} from the
// Chebyshev-Gauss-Lobatto points, w = 2 / (N (N+1) P_N^2); symmetrised.
void gll_nodes(int n, double *x, double *w) {
  if (n == 1) { x[0] = 0.0; w[0] = 2.0; return; }
  const int N = n - 1;
  for (int i = 0; i < n; ++i) {
    double xi = -std::cos(M_PI * i / N);
    for (int it = 0; it < 200; ++it) {
      double pm1, pN;
      legendre_pair(N, xi, &pm1, &pN);
      const double dx = (xi * pN - pm1) / ((N + 1.0) * pN);
      xi -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    double pm1, pN;
    legendre_pair(N, xi, &pm1, &pN);
    x[i] = xi;
    w[i] = 2.0 / (N * (N + 1.0) * pN * pN);
  }
  for (int i = 0; i < n / 2; ++i) {
    const double v = 0.5 * (x[N - i] - x[i]);
    const double ww = 0.5 * (w[N - i] + w[i]);
    x[i] = -v; x[N - i] = v;
    w[i] = ww; w[N - i] = ww;
  }
  if (n % 2) x[n / 2] = 0.0;
  x[0] = -1.0;
  x[N] = 1.0;
}

// Lagrange basis on arbitrary nodes, in the form of
// sum_factorization/include/math/lagrange_basis.hpp:29-65.
double lagrange_value(int n, const double *nodes, int j, double x) {
  double num = 1.0, den = 1.0;
  for (int m = 0; m < n; ++m) {
    if (m == j) continue;
    num *= (x - nodes[m]);
    den *= (nodes[j] - nodes[m]);
  }
  return num / den;
}

double lagrange_derivative(int n, const double *nodes, int j, double x) {
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

void derivative_matrix(int n, const double *nodes, double *D) {
  for (int q = 0; q < n; ++q)
    for (int b = 0; b < n; ++b) D[q * n + b] = lagrange_derivative(n, nodes, b, nodes[q]);
}

// -------------------------------------------------------------- box mesh --
__global__ void box_map_kernel(mfgb_box_desc b, uint32_t *__restrict__ map) {
  const int p = b.degree, n = p + 1, n3 = n * n * n;
  const int64_t Nx = (int64_t)p * b.nx + 1, Ny = (int64_t)p * b.ny + 1, Nz = (int64_t)p * b.nz + 1;
  const int64_t total = (int64_t)b.nx * b.ny * b.nz * n3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / n3;
    const int l = (int)(t - e * n3);
    const int i = l / (n * n), j = (l / n) % n, k = l % n;
    const int64_t cx = e % b.nx, cy = (e / b.nx) % b.ny, cz = e / ((int64_t)b.nx * b.ny);
    const int64_t gx = cx * p + k, gy = cy * p + j, gz = cz * p + i;
    const bool bnd = gx == 0 || gx == Nx - 1 || gy == 0 || gy == Ny - 1 || gz == 0 || gz == Nz - 1;
    map[t] = bnd ? MFGB_INVALID_DOF : (uint32_t)(gx + Nx * (gy + Ny * gz));
  }
}

cudaError_t box_map(const mfgb_box_desc &b, uint32_t *d_map, cudaStream_t s) {
  box_map_kernel<<<152 * 16, 256, 0, s>>>(b, d_map);
  return cudaGetLastError();
}

struct GeomParams {
  double x[10], w[10];    // target points / weights (GLL of the degree, or Gauss)
  double xg[9];           // GLL points of the geometry degree
  double V[90], Dv[90];   // V[i*ng+a] = l_a(x_i), Dv[i*ng+a] = l_a'(x_i) (geometry basis)
  int nt;                 // target points per direction
  int ng;                 // geometry points per direction
  int general;            // 0: targets are the geometry nodes (J by the square D)
  int nf[3], s;           // axis spans in fine-mesh units (BoxStride)
};

// fine-node range [a, b) of cell c on an axis of nf fine cells coarsened by s
__device__ __forceinline__ void axis_span(int64_t c, int nf, int s, double &a, double &w) {
  const int64_t lo = min(c * s, (int64_t)nf), hi = min((c + 1) * s, (int64_t)nf);
  a = (double)lo;
  w = (double)(hi - lo);
}

// One CTA per cell: the deformed geometry nodes (GLL points of the geometry
// degree) in shared memory, then J = dx/dxi at the operator's GLL points
// (the derivative matrix when both degrees agree, the tensor-product
// geometry basis otherwise, sum factorised through the dynamic shared arrays
// T1 [ng][ng][n] and T2 [ng][n][n], 3 components each) and
// G = |det J| w_i w_j w_k Jinv Jinv^T.
__global__ void box_geometry_kernel(mfgb_box_desc b, GeomParams gp, double *__restrict__ G,
                                    double *__restrict__ JxW) {
  __shared__ double xyz[729 * 3];
  extern __shared__ double sf[];
  __shared__ double s1[3][9];  // sin(2 pi X) of the cell's node coordinates, per axis
  const int n = gp.nt, n3 = n * n * n;
  const int ng = gp.ng, ng3 = ng * ng * ng;
  const int64_t e = blockIdx.x;
  const int64_t cx = e % b.nx, cy = (e / b.nx) % b.ny, cz = e / ((int64_t)b.nx * b.ny);
  const double hx = (b.hi[0] - b.lo[0]) / gp.nf[0], hy = (b.hi[1] - b.lo[1]) / gp.nf[1],
               hz = (b.hi[2] - b.lo[2]) / gp.nf[2];
  double ax, wx, ay, wy, az, wz;  // uniform box: a = c, w = 1 (the same bits as c + t)
  axis_span(cx, gp.nf[0], gp.s, ax, wx);
  axis_span(cy, gp.nf[1], gp.s, ay, wy);
  axis_span(cz, gp.nf[2], gp.s, az, wz);
  const double two_pi = 2.0 * M_PI;
  // the deformation is separable: 3 ng sines per cell instead of 3 ng^3
  if (threadIdx.x < 3 * ng) {
    const int d = threadIdx.x / ng, m = threadIdx.x % ng;
    const double t = 0.5 * (gp.xg[m] + 1.0);
    const double c = d == 0 ? b.lo[0] + (ax + t * wx) * hx
                            : d == 1 ? b.lo[1] + (ay + t * wy) * hy : b.lo[2] + (az + t * wz) * hz;
    s1[d][m] = sin(two_pi * c);
  }
  __syncthreads();
  for (int l = threadIdx.x; l < ng3; l += blockDim.x) {
    const int i = l / (ng * ng), j = (l / ng) % ng, k = l % ng;
    const double X = b.lo[0] + (ax + 0.5 * (gp.xg[k] + 1.0) * wx) * hx;
    const double Y = b.lo[1] + (ay + 0.5 * (gp.xg[j] + 1.0) * wy) * hy;
    const double Z = b.lo[2] + (az + 0.5 * (gp.xg[i] + 1.0) * wz) * hz;
    const double s = b.amplitude * s1[0][k] * s1[1][j] * s1[2][i];
    xyz[3 * l + 0] = X + s;
    xyz[3 * l + 1] = Y + s;
    xyz[3 * l + 2] = Z + s;
  }
  __syncthreads();
  // general: the geometry basis applied one direction at a time
  //   T1v = V_k x, T1d = Dv_k x; T2vv = V_j T1v, T2dv = Dv_j T1v, T2vd = V_j T1d
  //   J(:,r) = Dv_i T2vv, J(:,s) = V_i T2dv, J(:,t) = V_i T2vd
  const int t1 = ng * ng * n, t2 = ng * n * n;
  double *T1v = sf, *T1d = T1v + 3 * t1, *T2vv = T1d + 3 * t1, *T2dv = T2vv + 3 * t2,
         *T2vd = T2dv + 3 * t2;
  if (gp.general) {
    for (int l = threadIdx.x; l < t1; l += blockDim.x) {
      const int ab = l / n, k = l % n;
      double v0 = 0, v1 = 0, v2 = 0, d0 = 0, d1 = 0, d2 = 0;
      for (int c = 0; c < ng; ++c) {
        const double *x = xyz + 3 * (ab * ng + c);
        const double vk = gp.V[k * ng + c], dk = gp.Dv[k * ng + c];
        v0 += vk * x[0]; v1 += vk * x[1]; v2 += vk * x[2];
        d0 += dk * x[0]; d1 += dk * x[1]; d2 += dk * x[2];
      }
      T1v[3 * l] = v0; T1v[3 * l + 1] = v1; T1v[3 * l + 2] = v2;
      T1d[3 * l] = d0; T1d[3 * l + 1] = d1; T1d[3 * l + 2] = d2;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < t2; l += blockDim.x) {
      const int a = l / (n * n), j = (l / n) % n, k = l % n;
      double vv[3] = {0, 0, 0}, dv[3] = {0, 0, 0}, vd[3] = {0, 0, 0};
      for (int bb = 0; bb < ng; ++bb) {
        const int src = 3 * ((a * ng + bb) * n + k);
        const double vj = gp.V[j * ng + bb], dj = gp.Dv[j * ng + bb];
        for (int d = 0; d < 3; ++d) {
          vv[d] += vj * T1v[src + d];
          dv[d] += dj * T1v[src + d];
          vd[d] += vj * T1d[src + d];
        }
      }
      for (int d = 0; d < 3; ++d) {
        T2vv[3 * l + d] = vv[d];
        T2dv[3 * l + d] = dv[d];
        T2vd[3 * l + d] = vd[d];
      }
    }
    __syncthreads();
  }
  for (int l = threadIdx.x; l < n3; l += blockDim.x) {
    const int i = l / (n * n), j = (l / n) % n, k = l % n;
    double J[3][3];
    if (!gp.general) {
      for (int d = 0; d < 3; ++d) {
        double jr = 0, js = 0, jt = 0;
        for (int m = 0; m < n; ++m) {
          jr += gp.Dv[i * n + m] * xyz[3 * (m * n * n + j * n + k) + d];
          js += gp.Dv[j * n + m] * xyz[3 * (i * n * n + m * n + k) + d];
          jt += gp.Dv[k * n + m] * xyz[3 * (i * n * n + j * n + m) + d];
        }
        J[d][0] = jr; J[d][1] = js; J[d][2] = jt;
      }
    } else {
      for (int d = 0; d < 3; ++d) J[d][0] = J[d][1] = J[d][2] = 0.0;
      for (int a = 0; a < ng; ++a) {
        const int src = 3 * ((a * n + j) * n + k);
        const double va = gp.V[i * ng + a], da = gp.Dv[i * ng + a];
        for (int d = 0; d < 3; ++d) {
          J[d][0] += da * T2vv[src + d];
          J[d][1] += va * T2dv[src + d];
          J[d][2] += va * T2vd[src + d];
        }
      }
    }
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    double Ji[3][3];
    const double id = 1.0 / det;  // one FP64 division per point
    Ji[0][0] = c00 * id;
    Ji[1][0] = c01 * id;
    Ji[2][0] = c02 * id;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    const double jxw = fabs(det) * gp.w[i] * gp.w[j] * gp.w[k];
    if (JxW) JxW[e * n3 + l] = jxw;
    double *Gc = G + e * 6 * n3 + l;
    int c = 0;
    for (int a = 0; a < 3; ++a)
      for (int bb = a; bb < 3; ++bb) {
        double s = 0;
        for (int d = 0; d < 3; ++d) s += Ji[a][d] * Ji[bb][d];
        Gc[c * n3] = jxw * s;
        ++c;
      }
  }
}

// Gauss-Legendre points/weights (Newton on P_n from Chebyshev guesses), ascending
void gauss_nodes(int n, double *x, double *w) {
  for (int i = 0; i < n; ++i) {
    double xi = -std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 200; ++it) {
      double pm1, pn;
      legendre_pair(n, xi, &pm1, &pn);
      dp = n * (xi * pn - pm1) / (xi * xi - 1.0);
      const double dx = pn / dp;
      xi -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    double pm1, pn;
    legendre_pair(n, xi, &pm1, &pn);
    dp = n * (xi * pn - pm1) / (xi * xi - 1.0);
    x[i] = xi;
    w[i] = 2.0 / ((1.0 - xi * xi) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) {
    const double v = 0.5 * (x[n - 1 - i] - x[i]), ww = 0.5 * (w[n - 1 - i] + w[i]);
    x[i] = -v; x[n - 1 - i] = v;
    w[i] = ww; w[n - 1 - i] = ww;
  }
  if (n % 2) x[n / 2] = 0.0;
}

cudaError_t box_geometry(const mfgb_box_desc &b, const double *gll_x, const double *gll_w,
                         const double *D, double *d_G, cudaStream_t s, bool at_gauss,
                         const BoxStride *bs, double *d_JxW, int n_gauss) {
  GeomParams gp{};
  if (bs && bs->s > 1) {
    for (int d = 0; d < 3; ++d) gp.nf[d] = bs->nf[d];
    gp.s = bs->s;
    if ((b.nx != (gp.nf[0] + gp.s - 1) / gp.s) || (b.ny != (gp.nf[1] + gp.s - 1) / gp.s) ||
        (b.nz != (gp.nf[2] + gp.s - 1) / gp.s))
      return cudaErrorInvalidValue;
  } else {
    gp.nf[0] = b.nx; gp.nf[1] = b.ny; gp.nf[2] = b.nz;
    gp.s = 1;
  }
  const int n = at_gauss && n_gauss > 0 ? n_gauss : b.degree + 1;
  const int g = b.geometry_degree > 0 ? b.geometry_degree : b.degree;
  if (g < 1 || g > 8 || n > 10) return cudaErrorInvalidValue;
  gp.ng = g + 1;
  gp.nt = n;
  double tx[10], tw[10];  // target points: the GLL points, or the Gauss points
  if (at_gauss) gauss_nodes(n, tx, tw);
  else for (int i = 0; i < n; ++i) { tx[i] = gll_x[i]; tw[i] = gll_w[i]; }
  for (int i = 0; i < n; ++i) { gp.x[i] = tx[i]; gp.w[i] = tw[i]; }
  gp.general = !(gp.ng == n && !at_gauss);
  if (!gp.general) {
    for (int i = 0; i < n; ++i) gp.xg[i] = gll_x[i];
    for (int i = 0; i < n * n; ++i) gp.Dv[i] = D[i];
  } else {
    double wg[9];
    gll_nodes(gp.ng, gp.xg, wg);
    for (int i = 0; i < n; ++i)
      for (int a = 0; a < gp.ng; ++a) {
        gp.V[i * gp.ng + a] = lagrange_value(gp.ng, gp.xg, a, tx[i]);
        gp.Dv[i * gp.ng + a] = lagrange_derivative(gp.ng, gp.xg, a, tx[i]);
      }
  }
  const int64_t n_cells = (int64_t)b.nx * b.ny * b.nz;
  if (n_cells == 0) return cudaSuccess;
  const int pts = std::max(n * n * n, gp.ng * gp.ng * gp.ng);
  const int threads = ((pts + 31) / 32) * 32;
  // sum-factorisation arrays of the general path (at most 103 KB: ng = 9, n = 10),
  // beside the 17.5 KB static node array: above 48 KB in total the kernel needs
  // the larger dynamic limit
  const size_t smem =
      gp.general ? sizeof(double) * 3 * (2 * gp.ng * gp.ng * n + 3 * gp.ng * n * n) : 0;
  if (smem > 0) {
    cudaError_t e = cudaFuncSetAttribute(box_geometry_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  box_geometry_kernel<<<(unsigned)n_cells, threads > 256 ? 256 : threads, smem, s>>>(b, gp, d_G,
                                                                                      d_JxW);
  return cudaGetLastError();
}

// ------------------------------------------------------- G conversions --
__global__ void g_to_df_kernel(int64_t n, const double *__restrict__ G, float2 *__restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double g = G[t];
    const float hi = (float)g;
    out[t] = make_float2(hi, (float)(g - (double)hi));
  }
}

__global__ void g_to_f32_kernel(int64_t n, const double *__restrict__ G, float *__restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = (float)G[t];
}

cudaError_t g_to_df(int64_t n, const double *G, float2 *Gdf, cudaStream_t s) {
  g_to_df_kernel<<<152 * 16, 256, 0, s>>>(n, G, Gdf);
  return cudaGetLastError();
}

cudaError_t g_to_f32(int64_t n, const double *G, float *G32, cudaStream_t s) {
  g_to_f32_kernel<<<152 * 16, 256, 0, s>>>(n, G, G32);
  return cudaGetLastError();
}

// ------------------------------------------------------------- diagonal --
// A[l,l] of one cell, l = (i,j,k): for GLL collocation the basis gradient
// d_r phi_l at point (a,b,c) is D[a][i] delta_bj delta_ck, so
//   A_e[l,l] = sum_a Grr(a,j,k) D[a][i]^2 + sum_b Gss(i,b,k) D[b][j]^2
//            + sum_c Gtt(i,j,c) D[c][k]^2
//            + 2 (Grs D[i][i] D[j][j] + Grt D[i][i] D[k][k] + Gst D[j][j] D[k][k])(i,j,k).
struct DiagParams {
  double D[81];
};

__global__ void diagonal_kernel(int n, int64_t n_cells, const uint32_t *__restrict__ map,
                                const double *__restrict__ G, DiagParams dp,
                                double *__restrict__ diag) {
  const int n3 = n * n * n;
  const int64_t total = n_cells * n3;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t dof = map[t];
    if (dof == MFGB_INVALID_DOF) continue;
    const int64_t e = t / n3;
    const int q = (int)(t - e * n3);
    const int i = q / (n * n), j = (q / n) % n, k = q % n;
    const double *Ge = G + e * 6 * n3;
    double d = 0.0;
    for (int a = 0; a < n; ++a) {
      const double di = dp.D[a * n + i], dj = dp.D[a * n + j], dk = dp.D[a * n + k];
      d += Ge[0 * n3 + a * n * n + j * n + k] * di * di;
      d += Ge[3 * n3 + i * n * n + a * n + k] * dj * dj;
      d += Ge[5 * n3 + i * n * n + j * n + a] * dk * dk;
    }
    const double Dii = dp.D[i * n + i], Djj = dp.D[j * n + j], Dkk = dp.D[k * n + k];
    d += 2.0 * Ge[1 * n3 + q] * Dii * Djj;
    d += 2.0 * Ge[2 * n3 + q] * Dii * Dkk;
    d += 2.0 * Ge[4 * n3 + q] * Djj * Dkk;
    atomicAdd(diag + dof, d);
  }
}

cudaError_t diagonal_f64(int N, int64_t n_cells, const uint32_t *map, const double *G,
                         const double *D, double *diag, cudaStream_t s) {
  DiagParams dp;
  for (int i = 0; i < 81; ++i) dp.D[i] = i < N * N ? D[i] : 0.0;
  diagonal_kernel<<<152 * 16, 256, 0, s>>>(N, n_cells, map, G, dp, diag);
  return cudaGetLastError();
}

// Exact diagonal of the Gauss-point operator (the quantity deal.II's
// MatrixFreeTools::compute_diagonal returns for bp5_kokkos/benchmark.cc:218-251):
// for local DoF (a, b, c) of a cell, sum over the Gauss points q = (i, j, k) of
// grad(phi)^T G grad(phi) + JxW phi^2 with phi = B[i][a] B[j][b] B[k][c] and
// d phi / d xi_0 = (DG B)[i][a] B[j][b] B[k][c], etc.  One CTA per cell, one
// thread per local DoF; G and JxW of the cell staged in shared memory.
struct GaussDiagParams {
  double B[100], DB[100];  // B[q*n + a], DB = DG B  (q < nq, a < n)
};

// The diagonal entry of DoF (a, b, c) is a sum over the Gauss points (i, j, k)
// of seven terms (the six G components and the mass term), each a product of
// 1D weights: with r = DB_i B_j B_k, s = B_i DB_j B_k, t = B_i B_j DB_k (basis
// a, b, c; DB = DG B the derivative at the Gauss points)
//   G_rr r^2 + G_ss s^2 + G_tt t^2 + 2 (G_rs r s + G_rt r t + G_st s t) + JxW (B_i B_j B_k)^2.
// The kernel contracts the seven quadrature arrays one direction at a time
// (k -> c, j -> b, i -> a) with the squared / mixed 1D weights (bb = B^2,
// dd = DB^2, bd = B DB): O(nq^3 n) per cell instead of O(nq^3 n^3).  One CTA
// per cell; shared memory holds the weights, stage 1 [T][nq][nq][n] and
// stage 2 [T][nq][n][n].
__constant__ int kDiagKind[3][7] = {
    // rr  rs  rt  ss  st  tt  W     weight kind per direction: 0 bb, 1 dd, 2 bd
    {1, 2, 2, 0, 0, 0, 0},  // i
    {0, 2, 0, 1, 2, 0, 0},  // j
    {0, 0, 2, 0, 2, 1, 0},  // k
};
__constant__ double kDiagFactor[7] = {1.0, 2.0, 2.0, 1.0, 2.0, 1.0, 1.0};

__global__ void __launch_bounds__(256)
    diagonal_gauss_kernel(int N, int NQ, int64_t n_cells, const uint32_t *__restrict__ map,
                          const double *__restrict__ G, const double *__restrict__ JxW,
                          GaussDiagParams gp, double *__restrict__ diag) {
  extern __shared__ double sm[];
  const int NT = JxW ? 7 : 6;
  const int N2 = N * N, N3 = N2 * N, Q2 = NQ * NQ, Q3 = Q2 * NQ, QN = NQ * N;
  double *w = sm;                        // [3][nq][n]: bb, dd, bd
  double *S1 = w + 3 * QN;               // [T][nq][nq][n]  (i, j, c)
  double *S2 = S1 + NT * Q2 * N;         // [T][nq][n][n]   (i, b, c)
  for (int t = threadIdx.x; t < QN; t += blockDim.x) {
    const double b = gp.B[t], d = gp.DB[t];
    w[t] = b * b;
    w[QN + t] = d * d;
    w[2 * QN + t] = b * d;
  }
  __syncthreads();
  for (int64_t e = blockIdx.x; e < n_cells; e += gridDim.x) {
    for (int l = threadIdx.x; l < NT * Q2 * N; l += blockDim.x) {  // k -> c
      const int T = l / (Q2 * N), r = l - T * Q2 * N, ij = r / N, c = r - ij * N;
      const double *src = (T < 6 ? G + (e * 6 + T) * Q3 : JxW + e * Q3) + ij * NQ;
      const double *wk = w + kDiagKind[2][T] * QN + c;
      double acc = 0.0;
      for (int k = 0; k < NQ; ++k) acc += wk[k * N] * __ldg(src + k);
      S1[l] = acc;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < NT * NQ * N2; l += blockDim.x) {  // j -> b
      const int T = l / (NQ * N2), r = l - T * NQ * N2, i = r / N2, bc = r - i * N2;
      const int b = bc / N, c = bc - b * N;
      const double *wj = w + kDiagKind[1][T] * QN + b;
      const double *s1 = S1 + T * Q2 * N + i * NQ * N + c;
      double acc = 0.0;
      for (int j = 0; j < NQ; ++j) acc += wj[j * N] * s1[j * N];
      S2[l] = acc;
    }
    __syncthreads();
    for (int l = threadIdx.x; l < N3; l += blockDim.x) {  // i -> a, scatter
      const uint32_t dof = map[e * N3 + l];
      if (dof == MFGB_INVALID_DOF) continue;
      const int a = l / N2, bc = l - a * N2;
      double acc = 0.0;
      for (int T = 0; T < NT; ++T) {
        const double *wi = w + kDiagKind[0][T] * QN + a;
        const double *s2 = S2 + T * NQ * N2 + bc;
        double t = 0.0;
        for (int i = 0; i < NQ; ++i) t += wi[i * N] * s2[i * N2];
        acc += kDiagFactor[T] * t;
      }
      atomicAdd(diag + dof, acc);
    }
    __syncthreads();  // S1 / S2 are rewritten for the next cell
  }
}

cudaError_t diagonal_gauss(int N, int NQ, int64_t n_cells, const uint32_t *map, const double *G,
                           const double *JxW, const double *B, const double *DG, double *diag,
                           cudaStream_t s) {
  if (N < 2 || N > 9 || NQ < N || NQ > 10) return cudaErrorInvalidValue;
  GaussDiagParams gp{};
  for (int q = 0; q < NQ; ++q)
    for (int a = 0; a < N; ++a) {
      gp.B[q * N + a] = B[q * N + a];
      double d = 0.0;
      for (int m = 0; m < NQ; ++m) d += DG[q * NQ + m] * B[m * N + a];
      gp.DB[q * N + a] = d;
    }
  if (n_cells == 0) return cudaSuccess;
  const int NT = JxW ? 7 : 6;
  const size_t smem = sizeof(double) * (3 * NQ * N + NT * NQ * NQ * N + NT * NQ * N * N);
  if (smem > 48 * 1024) {  // at most 98 KB (nq = 10, n = 9, mass term)
    const cudaError_t e = cudaFuncSetAttribute(diagonal_gauss_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const unsigned grid = (unsigned)std::min<int64_t>(n_cells, 152 * 8);
  diagonal_gauss_kernel<<<grid, 256, smem, s>>>(N, NQ, n_cells, map, G, JxW, gp, diag);
  return cudaGetLastError();
}

// ----------------------------------------------------------- constraints --
__global__ void set_constrained_kernel(int64_t nc, const int64_t *__restrict__ c, double *v,
                                       double value) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nc;
       t += (int64_t)gridDim.x * blockDim.x)
    v[c[t]] = value;
}

__global__ void copy_constrained_kernel(int64_t nc, const int64_t *__restrict__ c,
                                        const double *__restrict__ src, double *dst) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nc;
       t += (int64_t)gridDim.x * blockDim.x)
    dst[c[t]] = src[c[t]];
}

__global__ void invert_diagonal_kernel(int64_t n, double *d) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double v = d[t];
    d[t] = v > 0.0 ? 1.0 / v : 1.0;
  }
}

static unsigned grid_for(int64_t n) {
  const int64_t g = (n + 255) / 256;
  return (unsigned)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

cudaError_t set_constrained(int64_t nc, const int64_t *c, double *v, double value, cudaStream_t s) {
  if (nc == 0) return cudaSuccess;
  set_constrained_kernel<<<grid_for(nc), 256, 0, s>>>(nc, c, v, value);
  return cudaGetLastError();
}

cudaError_t copy_constrained(int64_t nc, const int64_t *c, const double *src, double *dst,
                             cudaStream_t s) {
  if (nc == 0) return cudaSuccess;
  copy_constrained_kernel<<<grid_for(nc), 256, 0, s>>>(nc, c, src, dst);
  return cudaGetLastError();
}

cudaError_t invert_diagonal(int64_t n, double *d, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  invert_diagonal_kernel<<<grid_for(n), 256, 0, s>>>(n, d);
  return cudaGetLastError();
}

}  // namespace mfgb
