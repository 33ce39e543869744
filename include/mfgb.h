/*
 * mfgb.h -- C ABI of the GB300-native matrix-free BK5/BP5 Laplacian engine
 * (libmfgb.so).
 *
 * Plain pointers and sizes only.  Vector and array arguments named `d_*` are
 * device pointers owned by the caller; `h_*` are host pointers.  `stream` is a
 * cudaStream_t passed as void* (NULL = legacy default stream).  Every call
 * returns an mfgb_status and never exits or aborts; the text of the last error
 * of the calling thread is available from mfgb_last_error().
 *
 * Each entry point names the reference interface it replaces (paths relative
 * to the dealii-X/benchmarks project root).
 */
#ifndef MFGB_H
#define MFGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int mfgb_status;
enum {
  MFGB_OK = 0,
  MFGB_ERR_INVALID_ARG = 1,
  MFGB_ERR_OUT_OF_MEMORY = 2,
  MFGB_ERR_NOT_CONVERGED = 3,
  MFGB_ERR_TIMEOUT = 4,
  MFGB_ERR_NONFINITE = 5,
  MFGB_ERR_CUDA = 6,
  MFGB_ERR_UNSUPPORTED = 7,
  /* an input outside the range the double-float kernels without per-cell
     scaling carry at FP64 accuracy: the largest magnitude of a vector, or of a
     cell's geometric factors, outside [2^-40, 2^55] (use MFGB_ARITH_FP64) */
  MFGB_ERR_RANGE = 8
};

/* Arithmetic used inside the operator kernels (vectors stay FP64).
   MFGB_ARITH_FP64_DF computes with float pairs on the FP32 pipes (48
   significant bits; 1e-12 relative against FP64 on the operator).  On GLL
   collocation operators (shapes 5 / 6 of the kernel shape table, the default
   at every degree), their BK6 vector form (every component on its own), the
   Gauss p+1 Laplacian, its Helmholtz form and the BP3 operator every cell is
   scaled by a power of two, so any FP64 input range is carried (so are the
   kernel seams, per element, given a 16-byte aligned G).  Elsewhere (shapes
   0-4, seams given an unaligned G) inputs must lie
   in the window of MFGB_ERR_RANGE: the operator's own
   geometric factors are checked when their pairs are built (the call returns
   MFGB_ERR_RANGE), caller-supplied G and vectors of the seams on every call,
   and the source vectors of operator applications on the device (reported by
   mfgb_check_device_errors, which the solvers call). */
enum {
  MFGB_ARITH_FP64 = 0,    /* native FP64 (DFMA) */
  MFGB_ARITH_FP64_DF = 1, /* FP64-accurate double-float on the FP32 pipes */
  MFGB_ARITH_FP32 = 2,    /* FP32 operator on FP32 vectors (multigrid levels) */
  MFGB_ARITH_FP64_TC = 3  /* native FP64 on the tensor cores (mma m8n8k4 .f64):
                             mfgb_bk1_evector at degree 1..6 only */
};

#define MFGB_INVALID_DOF_INDEX 0xFFFFFFFFu

typedef struct mfgb_operator mfgb_operator;

/* Structured box mesh: nx*ny*nz hex cells of degree p with GLL nodes,
   every geometry node moved by x_d += amplitude*sin(2 pi x)sin(2 pi y)sin(2 pi z),
   Dirichlet u = 0 on the whole boundary, lexicographic DoF numbering (x fastest).
   The cell geometry is the Q_g interpolant of the deformed map at the GLL
   points of degree g = geometry_degree (0: g = degree); multigrid levels use
   the fine degree so coarse cells stay as accurate as the fine ones. */
typedef struct {
  int nx, ny, nz;
  int degree;
  double lo[3], hi[3];
  double amplitude;
  int geometry_degree;
} mfgb_box_desc;

typedef struct {
  int max_steps;    /* ReductionControl max_steps */
  double tol;       /* absolute tolerance */
  double reduce;    /* relative reduction of the initial residual */
  int arith;        /* MFGB_ARITH_* used for the operator inside the solve */
} mfgb_cg_control;

typedef struct {
  int steps;        /* last_step() */
  double initial;   /* initial_value() */
  double last;      /* last_value() */
  int converged;    /* 1 if the reduction criterion was met */
} mfgb_solve_info;

/* Thread layout of the operator kernel for (arith, degree): 0 = one thread per
   (j,k) column of an element, 1 = one thread per quadrature point, 2 = columns
   with the geometric factors prefetched by bulk TMA copies, 3 / 4 = shapes 0 /
   2 at an alternative number of cells per thread block (the autotuner's
   elements-per-block choice); for MFGB_ARITH_FP64_DF also 5 / 6 = the
   offset-accumulation kernel with per-cell scaling at the cells per block of
   shapes 2 / 4 (GLL operators; elsewhere they run as 2 / 4).  The library
   starts from a built-in table; the autotuner overrides it.  No
   counterpart in the reference (its launch shape is a compile-time choice,
   CEED_BK/src/BK5/templated_cuda_benchmark.cc:114-124). */
mfgb_status mfgb_set_kernel_shape(int arith, int degree, int shape);
mfgb_status mfgb_get_kernel_shape(int arith, int degree, int *shape);

/* Reads and clears the device error word: MFGB_ERR_TIMEOUT if a kernel gave
   up on a bulk-copy wait since the last check (its results are invalid),
   MFGB_ERR_RANGE if a double-float application without per-cell scaling was
   given a source vector outside its range. */
mfgb_status mfgb_check_device_errors(void *stream);

/* Test hooks for the failure paths (no counterpart in the reference, whose
   drivers exit on any error, CEED_BK/src/BK5/templated_cuda_benchmark.cc:9-27).
   mfgb_test_fail_allocation(n): the n-th device allocation of the library from
   this call on fails as if the device were out of memory (0 = off).
   mfgb_test_expire_copy_wait(n): the next n applications of the double-float
   GLL operator (the offset-accumulation kernel) arm their first geometric-
   factor copy wait without issuing the copy and give up after 1 ms, so the
   bounded wait runs out with nothing in flight: the result is void and
   mfgb_check_device_errors returns MFGB_ERR_TIMEOUT. */
mfgb_status mfgb_test_fail_allocation(int n);
mfgb_status mfgb_test_expire_copy_wait(int n);

const char *mfgb_status_string(mfgb_status s);
const char *mfgb_last_error(void);
int mfgb_version(void);

/* ---- operator set-up ---------------------------------------------------
 * Replaces the LaplaceOperatorBK35 constructor
 * (bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:97-121):
 * dof map with invalid entries for constrained DoFs (:294-384) and the
 * geometric factors G[cell][6][q] (:229-292), built on the device. */
mfgb_status mfgb_operator_create_box(const mfgb_box_desc *box, mfgb_operator **op);

/* The Gauss-quadrature form the reference runs (BP5 variant: QGauss(p+1),
   values interpolated from the GLL nodes, collocation gradient at the Gauss
   points; bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:114
   and bk3_kokkos_kernel.h:156-404), on the same box mesh.  Exactly
   integrated stiffness on affine cells. */
mfgb_status mfgb_operator_create_box_gauss(const mfgb_box_desc *box, mfgb_operator **op);

/* The Helmholtz operator of bp5_kokkos (Step64::HelmholtzOperator,
   bp5_kokkos/benchmark.cc:141-205): mass plus stiffness, (u, v) + (grad u,
   grad v), at QGauss(p+1) on GLL nodal values (:93-94, :179-191); same box
   mesh and Dirichlet rows.  mfgb_compute_diagonal gives its exact diagonal
   (the compute_diagonal of :218-251). */
mfgb_status mfgb_operator_create_box_helmholtz(const mfgb_box_desc *box, mfgb_operator **op);

/* BP3 on the same box mesh: the Laplacian at QGauss(p+2) on GLL nodal values
   (the CEED BP3 quadrature; CEED_bp/include/bk3_kokkos_kernel.h:146-354 is the
   reference's L-vector kernel for it, CEED_BK/include/kernels/BK3 its E-vector
   form), G[cell][6][(p+2)^3].  mfgb_compute_diagonal gives its exact diagonal. */
mfgb_status mfgb_operator_create_box_bp3(const mfgb_box_desc *box, mfgb_operator **op);

/* Same, from caller-provided host arrays (the deal.II set-up path):
   h_dof_map[cell*(p+1)^3 + l] (0xFFFFFFFF = constrained), h_G[cell][6][(p+1)^3]
   in the order rr, rs, rt, ss, st, tt, and the list of constrained DoFs. */
mfgb_status mfgb_operator_create(int degree, int64_t n_dofs, int64_t n_cells,
                                 const uint32_t *h_dof_map, const double *h_G,
                                 int64_t n_constrained, const int64_t *h_constrained,
                                 mfgb_operator **op);

mfgb_status mfgb_operator_destroy(mfgb_operator *op);

/* m() / n() and sizes (portable_laplace_operator_bk35.h:418-430) */
mfgb_status mfgb_operator_info(const mfgb_operator *op, int64_t *n_dofs, int64_t *n_cells,
                               int *degree, int64_t *n_constrained);

/* Copies the operator's map, geometric factors and constraint list to host
   arrays (any pointer may be NULL). */
mfgb_status mfgb_operator_export(const mfgb_operator *op, uint32_t *h_dof_map, double *h_G,
                                 int64_t *h_constrained);

/* ---- operator application ----------------------------------------------
 * vmult / Tvmult (portable_laplace_operator_bk35.h:123-167, :386-400):
 * dst = 0; dst += sum_cells P^T A_e P src (masked gather, atomic scatter);
 * dst[c] = src[c] on constrained DoFs (copy_constrained_values). */
mfgb_status mfgb_vmult(const mfgb_operator *op, double *d_dst, const double *d_src, int arith,
                       void *stream);

/* The two parts of vmult, for callers that schedule them (the deal.II cell
   loop, portable_laplace_operator_bk35.h:140-162, and copy_constrained_values,
   :166): d_dst += sum_cells P^T A_e P d_src (one kernel launch), and
   d_dst[c] = d_src[c] on the constrained DoFs. */
mfgb_status mfgb_vmult_add(const mfgb_operator *op, double *d_dst, const double *d_src, int arith,
                           void *stream);
mfgb_status mfgb_copy_constrained(const mfgb_operator *op, double *d_dst, const double *d_src,
                                  void *stream);

/* BK6/BP6 vector Laplacian: the scalar operator applied to ncomp = 3
   interleaved FP64 components (vec[3*dof + c]), constrained DoFs identity in
   every component.  The CEED BK6 definition (vector form of BK5); no
   counterpart kernel in the reference.  GLL operators only. */
mfgb_status mfgb_vmult_vector(const mfgb_operator *op, double *d_dst, const double *d_src,
                              int ncomp, int arith, void *stream);

/* vmult in FP32 arithmetic on FP32 vectors (the multigrid levels; the FP32
   copy of G is built on first use). */
mfgb_status mfgb_vmult_f32(const mfgb_operator *op, float *d_dst, const float *d_src, void *stream);

/* Kernel seam of BK3::Parallel::KokkosKernel_1D_Block
   (bakeoff_problems_dealii/include/bk3_kokkos_kernel.h:32-43) in the
   GLL-collocated form: accumulates sum_cells P^T A_e P src into d_dst (no
   zeroing, no constrained copy).  d_dbasis[q*(p+1)+b] = l_b'(x_q); d_G as above. */
mfgb_status mfgb_bk5_lvector(int degree, int64_t n_cells, const double *d_dbasis,
                             const double *d_G, const double *d_src, double *d_dst,
                             const uint32_t *d_dof_indices, int arith, void *stream);

/* E-vector kernel seam of BK5::Parallel::LaplaceOperator<T,nq>
   (CEED_BK/include/kernels/BK5/templated_cuda_kernels.cuh:11-14):
   out_e = D^T G_e D in_e for every element, d_G[e][6][(p+1)^3]. */
mfgb_status mfgb_bk5_evector(int degree, int64_t nelmt, const double *d_dbasis, const double *d_G,
                             const double *d_in, double *d_out, int arith, void *stream);

/* E-vector seam of BK1::Parallel::MassOperator<T,nq>
   (CEED_BK/include/kernels/BK1/templated_cuda_kernels.cuh:11-13), the CEED BK1
   mass operator with nq = degree + 2 points and nm = degree + 1 modes:
   out_e = B^T (JxW_e o (B x B x B) in_e); d_basis[q*nm + i], d_JxW[e][nq^3],
   d_in/d_out[e][nm^3], point and mode indices with direction 0 slowest (the
   reference serial kernel's order, CEED_BK/include/kernels/BK1/serial_kernels.hpp;
   its CUDA kernel indexes JxW with direction 2 slowest).  arith FP64, FP64_DF
   (offset double-float with every element's input and JxW scaled by a power of
   two: any FP64 range), or FP64_TC (degree 1..6: the six 1D contractions as 8x8x4 FP64 tensor-core
   tiles, one warp per element, the comparison of the reference's
   sum_factorization/include/kernels/BK1/templated_cuda_mma_kernels.cuh). */
mfgb_status mfgb_bk1_evector(int degree, int64_t nelmt, const double *d_basis, const double *d_JxW,
                             const double *d_in, double *d_out, int arith, void *stream);

/* E-vector seam of BK3::Parallel::LaplaceOperator<T,nq>
   (CEED_BK/include/kernels/BK3/templated_cuda_kernels.cuh:11-14), the CEED BK3
   Laplacian with interpolation: nq = degree + 2 points, d_basis[q*nm + i],
   collocation derivative d_dbasis[q*nq + m] at the points, d_G[e][6][nq^3]
   (rr rs rt ss st tt, the CUDA kernel's layout), d_in/d_out[e][nm^3]. */
mfgb_status mfgb_bk3_evector(int degree, int64_t nelmt, const double *d_basis,
                             const double *d_dbasis, const double *d_G, const double *d_in,
                             double *d_out, int arith, void *stream);

/* vmult on HOST vectors (the call a CPU-side caller of the reference makes):
   h_dst = A h_src with the copies inside the call.  On box operators the apply
   is pipelined over z-slabs of cells: the DoF planes a slab needs go up, its
   cells are applied, and the planes it completes come back while the next
   slab's planes arrive (three streams, ordered after prior work on `stream`;
   `stream` waits for the result).  Pinned host buffers are needed for the copies
   to overlap (pageable ones are copied synchronously by CUDA).  The operator
   keeps two device vectors for this call after the first use. */
mfgb_status mfgb_vmult_host(const mfgb_operator *op, double *h_dst, const double *h_src, int arith,
                            void *stream);
/* number of z-slabs of that pipeline (1..64; 0 = automatic: 16, each slab at
   least two cell layers) */
mfgb_status mfgb_set_host_pipeline(int slabs);

/* ---- diagonal -------------------------------------------------------------
 * compute_diagonal (bp5_kokkos/benchmark.cc:218-251): exact diagonal of the
 * operator (1 on constrained rows), then d -> (d > 0 ? 1/d : 1). */
mfgb_status mfgb_compute_diagonal(const mfgb_operator *op, double *d_diag, void *stream);
mfgb_status mfgb_invert_diagonal(int64_t n, double *d_diag, void *stream);

/* ---- right-hand side ------------------------------------------------------
 * b_i = 2*((x_i >> 11) * 2^-53) - 1 with x_i the i-th output of
 * mt19937_64(seed), i in DoF order; 0 on constrained DoFs. */
mfgb_status mfgb_rhs_uniform(const mfgb_operator *op, uint64_t seed, double *d_b, void *stream);

/* ---- conjugate gradients ---------------------------------------------------
 * SolverCG + ReductionControl (bp5_kokkos/benchmark.cc:355-378;
 * bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:263-287).
 * d_x holds the initial guess on entry.  d_inv_diag is the preconditioner:
 * NULL = PreconditionIdentity, else DiagonalMatrix with that (inverse
 * diagonal) vector.  Returns MFGB_ERR_NOT_CONVERGED (with *info filled) when
 * max_steps is reached. */
mfgb_status mfgb_cg_solve(const mfgb_operator *op, const double *d_b, double *d_x,
                          const double *d_inv_diag, const mfgb_cg_control *ctl,
                          mfgb_solve_info *info, void *stream);

/* Same solve without allocating any device memory (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc during a solve -- an
 * application whose own allocator owns the device memory, or a solver called
 * from inside another library's time loop -- the work vectors, reduction
 * partials and scalars live in a fixed file-scope device array sized for at
 * most MFGB_CG_NOALLOC_MAX_DOFS unknowns (about 25 MB, held on every GPU that
 * loads the library until the process exits).  Larger operators are rejected
 * with MFGB_ERR_UNSUPPORTED.  All calls share that array: calls whose work
 * overlaps on the GPU race and must be serialised by the caller.  The first
 * call on a device looks up the array's address; make it before any stream
 * capture. */
#define MFGB_CG_NOALLOC_MAX_DOFS 1048576
mfgb_status mfgb_cg_solve_noalloc(const mfgb_operator *op, const double *d_b, double *d_x,
                                  const double *d_inv_diag, const mfgb_cg_control *ctl,
                                  mfgb_solve_info *info, void *stream);

/* ---- multigrid preconditioner (no counterpart in the reference) ----------
 * Geometric p- and h-multigrid V-cycle for the structured box: p_fine ->
 * p_fine/2 -> ... -> 1 on the fine mesh, then Q1 on coarsened meshes while
 * the largest cell count exceeds coarse_cells (level l keeps the fine mesh
 * nodes min(k 2^l, n) of each axis: nested for any n);
 * Chebyshev(degree) around Jacobi on [lmax/smoothing_range, 1.2 lmax] with
 * lmax from eig_iterations power iterations; FP64 Jacobi-CG on the coarsest
 * level.  precision 32 runs the V-cycle (operators, smoother, transfers) in
 * FP32, precision 64 in FP64 (double-float operator arithmetic). */
typedef struct mfgb_mg mfgb_mg;
typedef struct {
  int precision;           /* 32 or 64 */
  int chebyshev_degree;    /* e.g. 5 */
  double smoothing_range;  /* lambda_max / lambda_min of the smoothing interval, e.g. 15 */
  int eig_iterations;      /* power iterations for lambda_max, e.g. 20 */
  int coarse_cells;        /* stop h-coarsening once max(nx,ny,nz) <= coarse_cells, e.g. 4 */
  double coarse_tol;       /* relative residual of the coarse Jacobi-CG, e.g. 1e-12 */
} mfgb_mg_params;

mfgb_status mfgb_mg_setup(const mfgb_box_desc *fine, const mfgb_mg_params *params, mfgb_mg **mg);
/* the same, with the finest level borrowing the caller's box operator (created
   by mfgb_operator_create_box; no second geometry set-up); the operator must
   outlive the hierarchy */
mfgb_status mfgb_mg_setup_shared(const mfgb_operator *fine_op, const mfgb_mg_params *params,
                                 mfgb_mg **mg);
mfgb_status mfgb_mg_destroy(mfgb_mg *mg);
/* level sizes (h_* arrays of n_levels entries, any may be NULL) */
mfgb_status mfgb_mg_info(const mfgb_mg *mg, int *n_levels, int64_t *h_dofs, int *h_degree,
                         double *h_lmax);
/* d_dst = M d_src: one V-cycle applied to an FP64 vector */
mfgb_status mfgb_mg_vmult(mfgb_mg *mg, double *d_dst, const double *d_src, void *stream);
/* FP64 PCG (SolverCG + ReductionControl semantics) with the V-cycle as the
   preconditioner; ctl->arith is the arithmetic of the outer operator. */
mfgb_status mfgb_mg_cg_solve(const mfgb_operator *op, mfgb_mg *mg, const double *d_b, double *d_x,
                             const mfgb_cg_control *ctl, mfgb_solve_info *info, void *stream);

/* Learned smoother weights on the finest level (no counterpart in the
   reference): the Chebyshev smoother's Jacobi diagonal becomes
   D~ = sum_cells w_e D_e with w_e > 0 per cell (D_e the cell matrix's
   diagonal); NULL restores the plain diagonal.  The V-cycle stays linear and
   SPD.  lambda_max of D~^-1 A is re-estimated. */
mfgb_status mfgb_mg_set_smoother_weights(mfgb_mg *mg, const double *d_cell_weights);

/* ---- batched solves (no counterpart in the reference) ---------------------
 * Many independent box problems (own cells, degree, deformation each) solved
 * together: FP64 CG with per-problem scalars and SolverCG/ReductionControl
 * semantics per problem, preconditioned by the FP32 multigrid V-cycle of
 * mfgb_mg_setup applied to every problem at once (params->precision must be
 * 32).  Vectors are the problems' DoF vectors concatenated in order
 * (h_offsets from mfgb_batch_info, n_problems + 1 entries).  The problems'
 * operators of one degree are applied by one kernel launch; one CG iteration
 * of the whole batch is one CUDA graph launch. */
typedef struct mfgb_batch mfgb_batch;
mfgb_status mfgb_batch_create(const mfgb_box_desc *boxes, int n_problems,
                              const mfgb_mg_params *params, mfgb_batch **batch);
mfgb_status mfgb_batch_destroy(mfgb_batch *batch);
/* any output may be NULL; h_depth_dofs has n_depths entries, h_levels
   n_problems (multigrid levels of each problem) */
mfgb_status mfgb_batch_info(const mfgb_batch *batch, int *n_problems, int64_t *h_offsets,
                            int *n_depths, int64_t *h_depth_dofs, int *h_levels);
/* b_i uniform in [-1, 1) from std::mt19937_64(h_seeds[i]), boundary DoFs 0 */
mfgb_status mfgb_batch_rhs_uniform(const mfgb_batch *batch, const uint64_t *h_seeds, double *d_b,
                                   void *stream);
/* d_dst = A d_src for every problem (FP64, double-float arithmetic) */
mfgb_status mfgb_batch_vmult(mfgb_batch *batch, double *d_dst, const double *d_src, void *stream);
/* d_dst = M d_src: one batched V-cycle */
mfgb_status mfgb_batch_precondition(mfgb_batch *batch, double *d_dst, const double *d_src,
                                    void *stream);
/* solves A_i x_i = b_i for every problem; h_info has n_problems entries.
   MFGB_ERR_NOT_CONVERGED if any problem reached max_steps (infos filled).
   Once the problems still running hold at most 75 % of the DoFs of the current
   launch plan, the union operators and tables are gathered again for them
   (converged problems stop costing work).  Each plan's iterations run as one
   CUDA graph launch: a conditional while node repeats one iteration until no
   problem runs, the running ones hold at most 75 % of the plan's DoFs, or
   max_steps iterations; the host only gathers the next plan. */
mfgb_status mfgb_batch_cg_solve(mfgb_batch *batch, const double *d_b, double *d_x,
                                const mfgb_cg_control *ctl, mfgb_solve_info *h_info, void *stream);
/* number of launch plans gathered during the last mfgb_batch_cg_solve */
mfgb_status mfgb_batch_last_solve_stats(const mfgb_batch *batch, int *n_replans);
/* number of graph launches of the last mfgb_batch_cg_solve (one per launch
   plan with the device-side loop; one per iteration where a CUDA driver cannot
   build the conditional graph) */
mfgb_status mfgb_batch_last_solve_launches(const mfgb_batch *batch, int *n_launches);

/* ---- learned part: features, targets, MLP (no counterpart in the reference)
 * features: per cell, dx/dxi at the 8 corner nodes (72 values, scaled by
 *   |mean corner det J|^(-1/3)) and p/8 -> float[n_cells][73] (box operators)
 * targets: lambda_max(D_e^-1 A_e) per cell by FP64 power iteration
 * MLP 73-64-64-1, relu, softplus output; parameters FP32 in the order
 *   W1[64][73], b1[64], W2[64][64], b2[64], w3[64], b3 (mfgb_mlp_n_params())
 * training: Adam on MSE, minibatches drawn by a fixed hash of (seed, step)
 * inference: BF16 tensor-core MMAs with FP32 accumulation */
int mfgb_mlp_n_params(void);
mfgb_status mfgb_cell_features(const mfgb_operator *op, float *d_features, void *stream);
mfgb_status mfgb_cell_lambda(const mfgb_operator *op, double *d_lambda, int iterations,
                             void *stream);
/* per-cell error reduction of one V-cycle of mg (the hierarchy of op's mesh),
   the multigrid's own training data for the smoother weights:
   rho_c = |E e|_c / |e|_c, E = I - M A, summed over n_vectors seeded random
   errors (U[-1,1] from mt19937_64(seed + k), 0 on Dirichlet DoFs) */
mfgb_status mfgb_cell_error_reduction(const mfgb_operator *op, mfgb_mg *mg, int n_vectors,
                                      uint64_t seed, double *d_rho, void *stream);
mfgb_status mfgb_mlp_loss_grad(const float *d_params, const float *d_X, const float *d_t, int n,
                               float *h_grad, float *h_loss);
mfgb_status mfgb_mlp_train(float *d_params, const float *d_X, const float *d_t, int64_t n,
                           int steps, int batch, float lr, uint64_t seed, float *h_loss);
mfgb_status mfgb_mlp_forward_f32(const float *d_params, const float *d_X, int n, float *d_y);
mfgb_status mfgb_mlp_infer(const float *d_params, const float *d_X, int64_t n, double *d_y,
                           void *stream);

/* ---- arithmetic-pipe throughput (no counterpart in the reference) --------
 * Floating-point operations per second of one arithmetic pipe on the current
 * GPU, from independent register-only chains on 8 CTAs of 256 threads per SM:
 * pipe 0 FP64 FMA, 1 FP32 FMA, 2 FP64 tensor-core MMA (mma.sync m8n8k4 f64, the
 * instruction of sum_factorization/include/kernels/BK1/cuda_mma_kernels.cuh:94-100),
 * 3 BF16 tensor-core mma.sync m16n8k16 with FP32 accumulation, 4 packed dual
 * FP32 FMA (fma.rn.f32x2), 5 / 6 scalar / packed FP32 FMAs with one integer
 * lop3 per FMA step (the lop3 counts nothing).  An FMA counts 2,
 * an m x n x k MMA 2 m n k.  The operator kernels' choice of arithmetic rests on
 * these rates. */
mfgb_status mfgb_pipe_rate(int pipe, int iters, int reps, double *ops_per_s);

/* Host link throughput with pinned host buffers of `bytes` (a multiple of 16):
 * mode 0 host->device, 1 device->host, 2 both directions at once, by the copy
 * engines; 3 / 4 / 5 the same by an SM copy kernel.  *bytes_per_s = bytes moved
 * (both directions summed) per second, best of `reps`.  The bound of
 * mfgb_vmult_host, which moves every DoF once each way. */
mfgb_status mfgb_link_rate(int mode, int64_t bytes, int reps, double *bytes_per_s);

/* ---- vector kernels used by the solver (exposed for tests) -------------- */
/* result[0] = sum a_i b_i (deterministic two-stage reduction) */
mfgb_status mfgb_dot(int64_t n, const double *d_a, const double *d_b, double *h_result,
                     void *stream);

#ifdef __cplusplus
}
#endif
#endif
