"""BP5 driver (the counterpart of the reference's solver drivers,
bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:263-313 and
bp5_kokkos/benchmark.cc:296-410): builds the deformed box problem, solves it
with the chosen method and prints one JSON line (iterations, residuals,
best-of-N solve time, apply time).

python -m benchmarks_gb300.bp5 --cells 128 128 64 --degree 4 --solver mg32
    solvers: mg32 (FP32 V-cycle in FP64 CG), mg64, jacobi, identity,
             helmholtz (bp5_kokkos's Helmholtz operator with Jacobi-PCG),
             batch (the seeded --problems mix solved together; --cells and
             --degree unused)
    --quadrature gll | gauss | bp3: the operator form (BP3: CEED_bp's
             q = p + 2 Laplacian, CEED_bp/include/bk3_kokkos_kernel.h:146-354)
"""
from __future__ import annotations

import argparse
import json
import time


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m benchmarks_gb300.bp5")
    ap.add_argument("--cells", type=int, nargs=3, default=[32, 32, 32])
    ap.add_argument("--degree", type=int, default=4)
    ap.add_argument("--amplitude", type=float, default=0.05)
    ap.add_argument("--solver", choices=["mg32", "mg64", "jacobi", "identity", "helmholtz",
                                         "batch"], default="mg32")
    ap.add_argument("--problems", type=int, default=256, help="batch: number of problems")
    ap.add_argument("--tol", type=float, default=1e-300, help="absolute tolerance")
    ap.add_argument("--reduce", type=float, default=1e-10, help="relative reduction")
    ap.add_argument("--max-steps", type=int, default=100000)
    ap.add_argument("--repeat", type=int, default=2, help="solves (best time reported)")
    ap.add_argument("--seed", type=int, default=1, help="right-hand side U[-1,1] seed")
    ap.add_argument("--arith", choices=["df", "fp64"], default="df")
    ap.add_argument("--quadrature", choices=["gll", "gauss", "bp3"], default="gll",
                    help="operator form: GLL collocation (BK5), Gauss p+1, BP3 (Gauss p+2)")
    a = ap.parse_args(argv)
    import torch

    import benchmarks_gb300 as mf
    torch.cuda.set_device(0)
    mesh = mf.BoxMesh(*a.cells, degree=a.degree, amplitude=a.amplitude)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    if a.solver == "batch":
        meshes, seeds = mf.batch_workload(a.problems, seed=2024)
        B, t_setup = timed(lambda: mf.BatchSolver(meshes))
        b = B.rhs_uniform(seeds)
        best = None
        for _ in range(max(1, a.repeat)):
            x = B.initialize_dof_vector()
            _, t = timed(lambda: B.solve(x, b, max_steps=200, reduce=a.reduce))
            best = t if best is None else min(best, t)
        steps = [i["steps"] for i in B.infos]
        print(json.dumps({"solver": "batch", "problems": a.problems, "n_dofs": B.n_dofs,
                          "setup_seconds": t_setup, "solve_seconds": best,
                          "iterations_min_max": [min(steps), max(steps)], "replans": B.replans}))
        return

    if a.solver == "helmholtz":
        A, t_setup = timed(lambda: mf.HelmholtzOperator(mesh, arith=a.arith))
    else:
        A, t_setup = timed(lambda: mf.LaplaceOperator(mesh, arith=a.arith,
                                                      quadrature=a.quadrature))
    if a.solver in ("mg32", "mg64"):
        P, t_pre = timed(lambda: mf.MGPreconditioner(mesh, precision=int(a.solver[2:]), operator=A))
    elif a.solver in ("jacobi", "helmholtz"):
        P, t_pre = timed(A.get_matrix_diagonal_inverse)
    else:
        P, t_pre = mf.PreconditionIdentity(), 0.0
    b = A.rhs_uniform(a.seed)
    best, info = None, {}
    for _ in range(max(1, a.repeat)):
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(a.max_steps, a.tol, a.reduce)
        converged = True

        def solve():
            try:
                mf.SolverCG(ctl).solve(A, x, b, P)
                return True
            except mf.MfgbError as e:
                if e.status != mf._abi.ERR_NOT_CONVERGED:
                    raise
                return False

        converged, t = timed(solve)
        best = t if best is None else min(best, t)
        info = {"iterations": ctl.last_step(), "initial_residual": ctl.initial_value(),
                "final_residual": ctl.last_value(), "converged": converged}
    y = A.initialize_dof_vector()
    _, t_apply = timed(lambda: [A.vmult(y, x) for _ in range(10)])
    print(json.dumps({"solver": a.solver, "cells": a.cells, "degree": a.degree,
                      "n_dofs": A.m(), "setup_seconds": t_setup, "preconditioner_seconds": t_pre,
                      "solve_seconds": best, **info, "vmult_seconds": t_apply / 10}))


if __name__ == "__main__":
    main()
