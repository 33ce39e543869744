// mfgb_operator.hpp -- header-only C++ adapter over the C ABI (mfgb.h) with the
// shape of the reference's operator/solver interface, so code written against
//   Portable::LaplaceOperatorBK35<dim, fe_degree, number>
//     (bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:16-95)
//   Step64::HelmholtzOperator::compute_diagonal / get_matrix_diagonal_inverse
//     (bp5_kokkos/benchmark.cc:153-168)
//   SolverCG<Vector>(ReductionControl).solve(A, x, b, P)
//     (bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:265-287)
// keeps its calls.  Vectors are mfgb::DeviceVector (device memory owned by the
// vector); errors throw mfgb::Error carrying the mfgb_status.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>

#include "mfgb.h"

namespace mfgb {

class Error : public std::runtime_error {
 public:
  Error(mfgb_status s, const std::string &msg) : std::runtime_error(msg), status(s) {}
  mfgb_status status;
};

inline void check(mfgb_status s) {
  if (s != MFGB_OK)
    throw Error(s, std::string(mfgb_status_string(s)) + ": " + mfgb_last_error());
}

// Minimal device vector (deal.II LinearAlgebra::distributed::Vector<double,
// MemorySpace::Default> on one rank): get_values(), size(), operator=(double).
class DeviceVector {
 public:
  DeviceVector() = default;
  explicit DeviceVector(int64_t n) { reinit(n); }
  ~DeviceVector() { cudaFree(ptr_); }
  DeviceVector(const DeviceVector &) = delete;
  DeviceVector &operator=(const DeviceVector &) = delete;
  DeviceVector(DeviceVector &&o) noexcept : ptr_(o.ptr_), n_(o.n_) { o.ptr_ = nullptr; o.n_ = 0; }

  void reinit(int64_t n) {
    cudaFree(ptr_);
    ptr_ = nullptr;
    n_ = n;
    if (n > 0 && cudaMalloc(&ptr_, sizeof(double) * n) != cudaSuccess)
      throw Error(MFGB_ERR_OUT_OF_MEMORY, "DeviceVector: cudaMalloc failed");
    *this = 0.0;
  }
  DeviceVector &operator=(double v) {
    if (v != 0.0) throw Error(MFGB_ERR_INVALID_ARG, "DeviceVector: only = 0 is supported");
    if (n_ && cudaMemset(ptr_, 0, sizeof(double) * n_) != cudaSuccess)
      throw Error(MFGB_ERR_CUDA, "DeviceVector: cudaMemset failed");
    return *this;
  }
  double *get_values() { return ptr_; }
  const double *get_values() const { return ptr_; }
  int64_t size() const { return n_; }
  int64_t locally_owned_size() const { return n_; }
  void copy_from_host(const double *h) {
    if (cudaMemcpy(ptr_, h, sizeof(double) * n_, cudaMemcpyHostToDevice) != cudaSuccess)
      throw Error(MFGB_ERR_CUDA, "DeviceVector: copy_from_host failed");
  }
  void copy_to_host(double *h) const {
    if (cudaMemcpy(h, ptr_, sizeof(double) * n_, cudaMemcpyDeviceToHost) != cudaSuccess)
      throw Error(MFGB_ERR_CUDA, "DeviceVector: copy_to_host failed");
  }
  double l2_norm() const {
    double r = 0;
    check(mfgb_dot(n_, ptr_, ptr_, &r, nullptr));
    return r > 0 ? __builtin_sqrt(r) : 0.0;
  }

 private:
  double *ptr_ = nullptr;
  int64_t n_ = 0;
};

class DiagonalMatrix {
 public:
  DeviceVector &get_vector() { return v_; }
  const DeviceVector &get_vector() const { return v_; }

 private:
  DeviceVector v_;
};

struct PreconditionIdentity {};

// The BK5 Laplacian (GLL collocation) on a structured box mesh or on caller
// arrays; `arith` selects native FP64 or FP64-accurate double-float kernels.
template <int dim, int fe_degree, typename number = double>
class LaplaceOperatorBK35 {
  static_assert(dim == 3, "only dim == 3");
  static_assert(fe_degree >= 1 && fe_degree <= 8, "fe_degree 1..8");

 public:
  explicit LaplaceOperatorBK35(mfgb_box_desc box, int arith = MFGB_ARITH_FP64_DF) : arith_(arith) {
    box.degree = fe_degree;
    mfgb_operator *op = nullptr;
    check(mfgb_operator_create_box(&box, &op));
    op_.reset(op);
    check(mfgb_operator_info(op, &n_dofs_, &n_cells_, nullptr, nullptr));
  }
  // deal.II set-up path: dof map with 0xFFFFFFFF on constrained DoFs,
  // G[cell][6][(p+1)^3], constrained DoF list
  LaplaceOperatorBK35(int64_t n_dofs, int64_t n_cells, const uint32_t *dof_map, const double *G,
                      int64_t n_constrained, const int64_t *constrained,
                      int arith = MFGB_ARITH_FP64_DF)
      : arith_(arith) {
    mfgb_operator *op = nullptr;
    check(mfgb_operator_create(fe_degree, n_dofs, n_cells, dof_map, G, n_constrained, constrained,
                               &op));
    op_.reset(op);
    n_dofs_ = n_dofs;
    n_cells_ = n_cells;
  }

  void vmult(DeviceVector &dst, const DeviceVector &src) const {
    check(mfgb_vmult(op_.get(), dst.get_values(), src.get_values(), arith_, nullptr));
  }
  void Tvmult(DeviceVector &dst, const DeviceVector &src) const { vmult(dst, src); }
  // vmult_dummy (portable_laplace_operator_bk35.h:170-225): computation_on runs
  // dst = 0 and the cell loop; ghost_exchange_on does the single-GPU part of the
  // exchange, the identity rows (compress and the ghost update are no-ops here)
  void vmult_dummy(DeviceVector &dst, const DeviceVector &src, bool ghost_exchange_on,
                   bool computation_on) const {
    if (computation_on) {
      if (cudaMemset(dst.get_values(), 0, sizeof(double) * dst.locally_owned_size()) != cudaSuccess)
        throw Error(MFGB_ERR_CUDA, "vmult_dummy: dst = 0");
      check(mfgb_vmult_add(op_.get(), dst.get_values(), src.get_values(), arith_, nullptr));
    }
    if (ghost_exchange_on)
      check(mfgb_copy_constrained(op_.get(), dst.get_values(), src.get_values(), nullptr));
  }
  // BK6: the operator on 3 interleaved components (vec[3 dof + c]; dst and src
  // hold 3 m() entries); GLL operators only
  void vmult_vector(DeviceVector &dst, const DeviceVector &src) const {
    check(mfgb_vmult_vector(op_.get(), dst.get_values(), src.get_values(), 3, arith_, nullptr));
  }
  // host vectors (pinned for overlap): copies pipelined with the apply; returns
  // after the result is in dst
  void vmult_host(double *dst, const double *src) const {
    check(mfgb_vmult_host(op_.get(), dst, src, arith_, nullptr));
    check(mfgb_check_device_errors(nullptr));
  }
  void initialize_dof_vector(DeviceVector &v) const { v.reinit(n_dofs_); }
  int64_t m() const { return n_dofs_; }
  int64_t n() const { return n_dofs_; }
  int64_t n_cells() const { return n_cells_; }

  void compute_diagonal() {
    inverse_diagonal_ = std::make_shared<DiagonalMatrix>();
    DeviceVector &d = inverse_diagonal_->get_vector();
    d.reinit(n_dofs_);
    check(mfgb_compute_diagonal(op_.get(), d.get_values(), nullptr));
    check(mfgb_invert_diagonal(n_dofs_, d.get_values(), nullptr));
  }
  std::shared_ptr<DiagonalMatrix> get_matrix_diagonal_inverse() const { return inverse_diagonal_; }

  // el(row, col) of bp5_kokkos (benchmark.cc:283-292): a diagonal entry, 1 / the
  // inverse diagonal of compute_diagonal(); only row == col is defined
  double el(int64_t row, int64_t col) const {
    if (row != col || row < 0 || row >= n_dofs_)
      throw std::invalid_argument("el: only diagonal entries inside the matrix");
    if (!inverse_diagonal_) throw std::logic_error("el: call compute_diagonal() first");
    double v = 0.0;
    if (cudaMemcpy(&v, inverse_diagonal_->get_vector().get_values() + row, sizeof(double),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      throw std::runtime_error("el: device read failed");
    return 1.0 / v;
  }

  const mfgb_operator *handle() const { return op_.get(); }
  int arith() const { return arith_; }

 protected:
  struct FromHandle {};
  LaplaceOperatorBK35(FromHandle, mfgb_operator *op, int arith) : arith_(arith) {
    op_.reset(op);
    check(mfgb_operator_info(op, &n_dofs_, &n_cells_, nullptr, nullptr));
  }
  static mfgb_operator *create(mfgb_status (*fn)(const mfgb_box_desc *, mfgb_operator **),
                               mfgb_box_desc box) {
    box.degree = fe_degree;
    mfgb_operator *op = nullptr;
    check(fn(&box, &op));
    return op;
  }

 private:
  struct Deleter {
    void operator()(mfgb_operator *p) const { mfgb_operator_destroy(p); }
  };
  std::unique_ptr<mfgb_operator, Deleter> op_;
  int64_t n_dofs_ = 0, n_cells_ = 0;
  int arith_;
  std::shared_ptr<DiagonalMatrix> inverse_diagonal_;
};

// Step64::HelmholtzOperator of bp5_kokkos (benchmark.cc:141-251): mass +
// stiffness at QGauss(p+1), same interface (vmult, compute_diagonal,
// get_matrix_diagonal_inverse, ...)
template <int dim, int fe_degree, typename number = double>
class HelmholtzOperator : public LaplaceOperatorBK35<dim, fe_degree, number> {
  using Base = LaplaceOperatorBK35<dim, fe_degree, number>;

 public:
  explicit HelmholtzOperator(mfgb_box_desc box, int arith = MFGB_ARITH_FP64_DF)
      : Base(typename Base::FromHandle{}, Base::create(mfgb_operator_create_box_helmholtz, box),
             arith) {}
};

// The BP3 Laplacian (QGauss(p+2) on GLL nodal values)
template <int dim, int fe_degree, typename number = double>
class LaplaceOperatorBP3 : public LaplaceOperatorBK35<dim, fe_degree, number> {
  using Base = LaplaceOperatorBK35<dim, fe_degree, number>;

 public:
  explicit LaplaceOperatorBP3(mfgb_box_desc box, int arith = MFGB_ARITH_FP64_DF)
      : Base(typename Base::FromHandle{}, Base::create(mfgb_operator_create_box_bp3, box), arith) {}
};

// V-cycle preconditioner (mfgb_mg_*), FP32 or FP64
class MGPreconditioner {
 public:
  MGPreconditioner(const mfgb_box_desc &box, int precision = 32) {
    mfgb_mg_params prm{precision, 5, 15.0, 20, 4, 1e-12};
    mfgb_mg *mg = nullptr;
    check(mfgb_mg_setup(&box, &prm, &mg));
    mg_.reset(mg);
  }
  void vmult(DeviceVector &dst, const DeviceVector &src) const {
    check(mfgb_mg_vmult(mg_.get(), dst.get_values(), src.get_values(), nullptr));
  }
  mfgb_mg *handle() const { return mg_.get(); }

 private:
  struct Deleter {
    void operator()(mfgb_mg *p) const { mfgb_mg_destroy(p); }
  };
  std::unique_ptr<mfgb_mg, Deleter> mg_;
};

class ReductionControl {
 public:
  ReductionControl(int max_steps = 100, double tol = 1e-10, double reduce = 1e-2)
      : max_steps_(max_steps), tol_(tol), reduce_(reduce) {}
  int last_step() const { return info_.steps; }
  double initial_value() const { return info_.initial; }
  double last_value() const { return info_.last; }
  mfgb_cg_control control(int arith) const { return {max_steps_, tol_, reduce_, arith}; }
  mfgb_solve_info &info() { return info_; }

 private:
  int max_steps_;
  double tol_, reduce_;
  mfgb_solve_info info_{};
};

// SolverCG: throws Error with status MFGB_ERR_NOT_CONVERGED where deal.II
// throws SolverControl::NoConvergence (bp5_kokkos/benchmark.cc:366-374).
class SolverCG {
 public:
  explicit SolverCG(ReductionControl &c) : control_(c) {}

  template <class Op>
  void solve(const Op &A, DeviceVector &x, const DeviceVector &b, const PreconditionIdentity &) {
    const mfgb_cg_control ctl = control_.control(A.arith());
    check(mfgb_cg_solve(A.handle(), b.get_values(), x.get_values(), nullptr, &ctl,
                        &control_.info(), nullptr));
  }
  template <class Op>
  void solve(const Op &A, DeviceVector &x, const DeviceVector &b, const DiagonalMatrix &P) {
    const mfgb_cg_control ctl = control_.control(A.arith());
    check(mfgb_cg_solve(A.handle(), b.get_values(), x.get_values(), P.get_vector().get_values(),
                        &ctl, &control_.info(), nullptr));
  }
  template <class Op>
  void solve(const Op &A, DeviceVector &x, const DeviceVector &b, const MGPreconditioner &P) {
    const mfgb_cg_control ctl = control_.control(A.arith());
    check(mfgb_mg_cg_solve(A.handle(), P.handle(), b.get_values(), x.get_values(), &ctl,
                           &control_.info(), nullptr));
  }

 private:
  ReductionControl &control_;
};

}  // namespace mfgb
