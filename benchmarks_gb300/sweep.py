"""Degree x size sweep of the BK5 / BP5 workload on one GPU: operator apply
GDoF/s (double-float, device vectors), BK6 apply GDoF/s and Jacobi-CG to a
relative reduction of 1e-10 on structured deformed boxes, the reference's
scaling study restated for this engine
(bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:263-313:
best-of repetitions of back-to-back applies, CG to a reduction).

python -m benchmarks_gb300.sweep [--degrees 1 .. 8] [--dofs 1e5 1e6 1e7 1.5e8]
    [--cg-max-dofs 1e7] [--bk6-dofs 1e7] [--reps 10]

One JSON line per (degree, size).  The mesh has n x n x n cells with
n = round((N^(1/3) - 1) / p), amplitude 0.05, seeded U[-1,1] right-hand side.
"""
from __future__ import annotations

import argparse
import json


def _mesh(mf, degree, target):
    n = max(2, round((target ** (1.0 / 3.0) - 1) / degree))
    return mf.BoxMesh(n, n, n, degree=degree, amplitude=0.05), n


def _time_apply(torch, fn, reps):
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run(degrees, sizes, cg_max_dofs, bk6_sizes, reps, emit=print):
    import torch

    import benchmarks_gb300 as mf
    rows = []
    for p in degrees:
        for target in sizes:
            mesh, n = _mesh(mf, p, target)
            A = mf.LaplaceOperator(mesh)
            N = A.m()
            row = {"degree": p, "cells": [n, n, n], "n_dofs": N}
            x = A.rhs_uniform(1)
            y = A.initialize_dof_vector()
            ms = _time_apply(torch, lambda: A.vmult(y, x), reps)
            row.update(apply_ms=ms, apply_gdofs=N / ms / 1e6)
            if any(abs(target - s) <= 1e-6 * s for s in bk6_sizes):
                xv = torch.rand(3 * N, dtype=torch.float64, device="cuda")
                yv = torch.zeros_like(xv)
                ms6 = _time_apply(torch, lambda: A.vmult_vector(yv, xv), reps)
                row.update(bk6_ms=ms6, bk6_gdofs=3 * N / ms6 / 1e6)
                del xv, yv
            if N <= cg_max_dofs:
                P = A.get_matrix_diagonal_inverse()
                ctl = mf.ReductionControl(1000000, 1e-300, 1e-10)
                xs = A.initialize_dof_vector()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                mf.SolverCG(ctl).solve(A, xs, x, P)
                e1.record()
                torch.cuda.synchronize()
                row.update(jacobi_cg_iterations=ctl.last_step(),
                           jacobi_cg_seconds=e0.elapsed_time(e1) / 1e3)
            rows.append(row)
            emit(json.dumps(row))
            del A, x, y
            torch.cuda.empty_cache()
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m benchmarks_gb300.sweep")
    ap.add_argument("--degrees", type=int, nargs="+", default=list(range(1, 9)))
    ap.add_argument("--dofs", type=float, nargs="+", default=[1e5, 1e6, 1e7, 1.5e8])
    ap.add_argument("--cg-max-dofs", type=float, default=1.2e7,
                    help="run Jacobi-CG to 1e-10 up to this many DoFs")
    ap.add_argument("--bk6-dofs", type=float, nargs="*", default=[1e7],
                    help="target sizes at which BK6 is timed too")
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    run(a.degrees, a.dofs, a.cg_max_dofs, a.bk6_dofs, a.reps)


if __name__ == "__main__":
    main()
