// bp5_solve.cc -- the reference's BP5 scaling driver shape
// (bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:245-328)
// written against the header-only adapter include/mfgb_operator.hpp: set up the
// operator on a deformed box, a seeded right-hand side, time best-of-5 batches
// of vmult and a CG solve, print one row of the reference's convergence table
// (cells dofs matvec CG_tot_time CG_time/iters cg_its cg_reduction).
//
// usage: bp5_solve nx ny nz [precond: none|jacobi|mg32|mg64|helmholtz] [reduce]
//   helmholtz: bp5_kokkos's Helmholtz operator with Jacobi-PCG
//   (bp5_kokkos/benchmark.cc:296-410); the table then describes that operator.
// A last line compares the host-buffer apply (vmult_host) with the device one.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "mfgb_operator.hpp"

using Clock = std::chrono::steady_clock;

int main(int argc, char **argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s nx ny nz [none|jacobi|mg32|mg64] [reduce]\n", argv[0]);
    return 1;
  }
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
  const std::string precond = argc > 4 ? argv[4] : "jacobi";
  const double reduce = argc > 5 ? std::atof(argv[5]) : 1e-10;
  try {
    mfgb_box_desc box{nx, ny, nz, 4, {0, 0, 0}, {1, 1, 1}, 0.05, 0};
    mfgb::LaplaceOperatorBK35<3, 4, double> A(box);
    mfgb::DeviceVector x, b, y;
    A.initialize_dof_vector(x);
    A.initialize_dof_vector(b);
    A.initialize_dof_vector(y);
    mfgb::check(mfgb_rhs_uniform(A.handle(), 1, b.get_values(), nullptr));

    double best_mv = 1e30;
    for (int rep = 0; rep < 5; ++rep) {
      const int n_mv = A.m() < 10000000 ? 200 : 50;
      cudaDeviceSynchronize();
      const auto t0 = Clock::now();
      for (int i = 0; i < n_mv; ++i) A.vmult(y, b);
      cudaDeviceSynchronize();
      best_mv = std::min(best_mv, std::chrono::duration<double>(Clock::now() - t0).count() / n_mv);
    }

    mfgb::ReductionControl control(1000000, 1e-300, reduce);
    mfgb::SolverCG cg(control);
    cudaDeviceSynchronize();
    auto t0 = Clock::now();
    double el_mid = 0.0;
    if (precond == "none") {
      cg.solve(A, x, b, mfgb::PreconditionIdentity());
    } else if (precond == "jacobi") {
      A.compute_diagonal();
      el_mid = A.el(A.m() / 2, A.m() / 2);  // bp5_kokkos's el(row, row)
      t0 = Clock::now();
      cg.solve(A, x, b, *A.get_matrix_diagonal_inverse());
    } else if (precond == "helmholtz") {
      mfgb::HelmholtzOperator<3, 4, double> H(box);
      H.compute_diagonal();
      t0 = Clock::now();
      cg.solve(H, x, b, *H.get_matrix_diagonal_inverse());
    } else {
      mfgb::MGPreconditioner mg(box, precond == "mg32" ? 32 : 64);
      cg.solve(A, x, b, mg);
    }
    cudaDeviceSynchronize();
    const double t_cg = std::chrono::duration<double>(Clock::now() - t0).count();
    const int its = control.last_step();
    const double red = its ? std::pow(control.last_value() / control.initial_value(), 1.0 / its) : 0.0;
    std::printf("cells dofs matvec CG_tot_time CG_time/iters cg_its cg_reduction\n");
    std::printf("%lld %lld %.3e %.3e %.3e %d %.3e\n", (long long)A.n_cells(), (long long)A.m(),
                best_mv, t_cg, its ? t_cg / its : 0.0, its, red);
    std::printf("GDoF/s %.3f\n", A.m() / best_mv * 1e-9);
    if (el_mid != 0.0) std::printf("el_mid %.17e\n", el_mid);
    // the host-buffer apply against the device apply (pinned host vectors)
    double *hs = nullptr, *hd = nullptr;
    const size_t bytes = sizeof(double) * A.m();
    if (cudaMallocHost((void **)&hs, bytes) != cudaSuccess ||
        cudaMallocHost((void **)&hd, bytes) != cudaSuccess)
      throw mfgb::Error(MFGB_ERR_OUT_OF_MEMORY, "pinned host vectors");
    cudaMemcpy(hs, b.get_values(), bytes, cudaMemcpyDeviceToHost);
    A.vmult(y, b);
    A.vmult_host(hd, hs);
    cudaMemcpy(hs, y.get_values(), bytes, cudaMemcpyDeviceToHost);
    double num = 0.0, den = 0.0;
    for (int64_t i = 0; i < A.m(); ++i) {
      num += (hd[i] - hs[i]) * (hd[i] - hs[i]);
      den += hs[i] * hs[i];
    }
    std::printf("host_apply_rel_diff %.3e\n", std::sqrt(num / den));
    cudaFreeHost(hs);
    cudaFreeHost(hd);
  } catch (const mfgb::Error &e) {
    std::fprintf(stderr, "mfgb error %d: %s\n", e.status, e.what());
    return 2;
  }
  return 0;
}
