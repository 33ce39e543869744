/*
 * mf_oracle.h -- CPU ORACLE for the BK5/BP5 matrix-free Laplacian.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links or calls
 * this code; it is used by tests/, by the smoke check and by the CPU-baseline
 * leg of bench.py, always as the checker and never as the thing measured on
 * the GPU path.
 *
 * It is a plain-C (FP64, optional OpenMP) restatement of the reference's
 * algorithm for the hot path.  Each function cites the reference file:line it
 * follows (paths relative to the dealii-X/benchmarks project root).
 *
 * Conventions (shared with the CUDA library):
 *   n = p + 1 points per direction, element-local index l = i*n*n + j*n + k
 *   (i slowest).  Reference directions r,s,t contract over i,j,k; on the box
 *   mesh k runs along x, j along y, i along z.  D[point*n + basis] = l_basis'
 *   (x_point) (the CEED_BK `dbasis` layout).  Geometric factors are stored
 *   G[cell][c][q] with c = (rr, rs, rt, ss, st, tt)
 *   (bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:266-287).
 *   The element-to-DoF map is map[cell*n^3 + l], 0xFFFFFFFF for constrained
 *   DoFs (portable_laplace_operator_bk35.h:335-375).
 */
#ifndef MF_ORACLE_H
#define MF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INVALID_DOF 0xFFFFFFFFu

/* ---- 1D bases ---------------------------------------------------------- */
void orc_gll(int n, double *x, double *w);
void orc_gauss(int n, double *x, double *w);
double orc_lagrange_value(int n, const double *nodes, int j, double x);
double orc_lagrange_derivative(int n, const double *nodes, int j, double x);
void orc_derivative_matrix(int n, const double *nodes, double *D);
void orc_interpolation_matrix(int n_from, const double *nodes_from, int n_to,
                              const double *pts_to, double *B);

/* ---- structured box mesh (Q_p, GLL nodes, sinusoidal deformation) ------ */
typedef struct {
  int nx, ny, nz;     /* cells per direction */
  int degree;         /* p */
  double lo[3], hi[3];/* box corners */
  double amplitude;   /* x_d += a sin(2 pi x) sin(2 pi y) sin(2 pi z) */
  int geometry_degree;/* Q_g geometry from the deformed GLL nodes of degree g (0: g = degree) */
  int stride;         /* coarsened level (> 1): cell c of an axis spans the nodes */
  int nf[3];          /* [min(c s, nf), min((c+1) s, nf)] of a uniform nf-cell axis;
                         nx = ceil(nf[0] / s) etc.  0 / 1: the uniform box itself */
} orc_box;

int64_t orc_box_n_dofs(const orc_box *b);
int64_t orc_box_n_cells(const orc_box *b);
/* node coordinates of cell e at the (g+1)^3 GLL points of the geometry degree
   g: xyz[l*3 + d] */
void orc_box_cell_nodes(const orc_box *b, int64_t cell, double *xyz);
/* element-to-DoF map (constrained -> ORC_INVALID_DOF) and constrained list.
   Returns the number of constrained DoFs; `constrained` may be NULL. */
int64_t orc_box_dof_map(const orc_box *b, uint32_t *map, int64_t *constrained);
/* G[cell][6][n^3] for every cell; returns number of cells with det J <= 0 */
int64_t orc_box_geometry(const orc_box *b, double *G);
/* Geometric factors of one cell from its node coordinates (same degree). */
int orc_cell_geometry(int n, const double *D, const double *w,
                      const double *xyz, double *Gcell);
/* Geometric factors at the n^3 GLL points from geometry nodes of another
   degree: V[i*ng + a] = l_a(x_i), Dv[i*ng + a] = l_a'(x_i). */
int orc_cell_geometry_general(int n, int ng, const double *V, const double *Dv,
                              const double *w, const double *xyz, double *Gcell);

/* ---- operator ------------------------------------------------------------ */
/* E-vector BK5: out_e = D^T G_e D in_e for every element (no gather) */
void orc_bk5_evector(int n, int64_t nelmt, const double *D, const double *G,
                     const double *in, double *out);
/* L-vector vmult: dst = sum_e P_e^T A_e P_e src, identity rows on constrained */
void orc_bk5_apply(int n, int64_t n_cells, const uint32_t *map, const double *D,
                   const double *G, int64_t n_dofs, int64_t n_constrained,
                   const int64_t *constrained, const double *src, double *dst);
/* exact diagonal of the L-vector operator (1 on constrained rows) */
void orc_bk5_diagonal(int n, int64_t n_cells, const uint32_t *map, const double *D,
                      const double *G, int64_t n_dofs, int64_t n_constrained,
                      const int64_t *constrained, double *diag);
/* diag -> inverse with the d <= 0 -> 1 guard */
void orc_invert_diagonal(int64_t n, double *d);

/* ---- Gauss-quadrature (BP5-variant / BP3) operator ------------------------
 * The deal.II-kernel form of the reference
 * (bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:156-228 interpolate GLL
 * nodal values to nq Gauss points per direction, :230-302 collocation gradient
 * at the Gauss points and metric apply, :305-334 transpose, :340-404
 * interpolate back).  B[q*n + i] = l_i(g_q) (GLL basis at Gauss points),
 * DG[q*nq + m] = L_m'(g_q) (Lagrange basis on the Gauss points);
 * Gg[cell][6][nq^3] from orc_box_geometry_gauss. */
typedef struct {
  int n, nq;                 /* GLL points, Gauss points per direction */
  const double *B, *DG;
} orc_gauss_basis;
/* B, DG (n <= 9, nq <= 10) for degree p and nq Gauss points */
void orc_gauss_basis_matrices(int p, int nq, double *B, double *DG);
/* G at the nq^3 Gauss points (Gauss weights) of every box cell */
int64_t orc_box_geometry_gauss(const orc_box *b, int nq, double *Gg);
/* the same, also JxW[cell][nq^3] at the Gauss points (JxW may be NULL) */
int64_t orc_box_geometry_gauss_jxw(const orc_box *b, int nq, double *Gg, double *JxW);
/* b_i = int phi_i f dx, f = 1, by the nq-point Gauss rule; 0 on constrained */
void orc_box_rhs_unit_gauss(const orc_box *b, int nq, int64_t n_constrained,
                            const int64_t *constrained, double *rhs);
/* CEED BK3 / BK1 E-vector operators: nm modes, nq points (nq = nm + 1 in the
   reference), basis[q*nm + i], dbasis[q*nq + m], G[e][6][nq^3], JxW[e][nq^3],
   in/out [e][nm^3]; point and mode indices with direction 0 slowest */
void orc_bk3_evector(int nm, int nq, int64_t nelmt, const double *basis, const double *dbasis,
                     const double *G, const double *in, double *out);
void orc_bk1_evector(int nm, int nq, int64_t nelmt, const double *basis, const double *JxW,
                     const double *in, double *out);
void orc_bk5g_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                    const uint32_t *map, const double *Gg, int64_t n_dofs,
                    int64_t n_constrained, const int64_t *constrained, const double *src,
                    double *dst);

/* ---- right-hand side ----------------------------------------------------- */
uint64_t orc_mt19937_64_nth(uint64_t seed, int64_t nth);
void orc_rhs_uniform(uint64_t seed, int64_t n_dofs, int64_t n_constrained,
                     const int64_t *constrained, double *b);

/* ---- solver -------------------------------------------------------------- */
typedef struct {
  int max_steps;
  double tol;     /* absolute tolerance */
  double reduce;  /* relative reduction */
} orc_reduction_control;

typedef struct {
  int steps;          /* last_step() */
  double initial;     /* initial_value() */
  double last;        /* last_value() */
  int converged;      /* 1 = success, 0 = failure (max steps / NaN) */
} orc_solve_info;

/* CG on any operator given as a callback (dst = A src) */
typedef void (*orc_apply_fn)(void *ctx, const double *src, double *dst);
orc_solve_info orc_cg_solve_op(orc_apply_fn apply, void *ctx, int64_t n_dofs,
                               const double *diag_inv, const double *b, double *x,
                               orc_reduction_control ctl);
/* CG on the Gauss-quadrature operator (PreconditionIdentity if diag_inv NULL) */
/* Helmholtz form of bp5_kokkos (mass + stiffness at the Gauss points): apply,
   exact diagonal (JxW NULL: the stiffness alone; 1 on constrained rows), CG */
void orc_helmholtz_apply(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                         const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                         int64_t n_constrained, const int64_t *constrained, const double *src,
                         double *dst);
void orc_gauss_diagonal(int n, int nq, const double *B, const double *DG, int64_t n_cells,
                        const uint32_t *map, const double *Gg, const double *JxW, int64_t n_dofs,
                        int64_t n_constrained, const int64_t *constrained, double *diag);
orc_solve_info orc_cg_solve_helmholtz(int n, int nq, const double *B, const double *DG,
                                      int64_t n_cells, const uint32_t *map, const double *Gg,
                                      const double *JxW, int64_t N, int64_t n_constrained,
                                      const int64_t *constrained, const double *diag_inv,
                                      const double *b, double *x, orc_reduction_control ctl);
orc_solve_info orc_cg_solve_gauss(int n, int nq, const double *B, const double *DG,
                                  int64_t n_cells, const uint32_t *map, const double *Gg,
                                  int64_t n_dofs, int64_t n_constrained,
                                  const int64_t *constrained, const double *diag_inv,
                                  const double *b, double *x, orc_reduction_control ctl);

/* Jacobi- (diag_inv != NULL) or identity-preconditioned CG on the BK5 operator */
orc_solve_info orc_cg_solve(int n, int64_t n_cells, const uint32_t *map,
                            const double *D, const double *G, int64_t n_dofs,
                            int64_t n_constrained, const int64_t *constrained,
                            const double *diag_inv, const double *b, double *x,
                            orc_reduction_control ctl);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
