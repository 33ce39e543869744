"""Parity with the CPU oracle at the benchmark's own configurations.

* The bench workload itself: p = 4 on 128 x 128 x 64 deformed cells (67,634,433
  DoFs, amplitude 0.05), seeded U[-1,1] src, both FP64 arithmetics, relative
  2-norm error <= 1e-12 (the operator's FP64 bar).
* The degree sweep's largest meshes (about 1.5e8 DoFs): p = 1 on 530^3 cells,
  where cell * 6 * n^3 passes 2^31, and p = 8 on 66^3 cells.
* Plain Jacobi-CG to a 1e-10 relative residual for p = 1..8 at about 1e5 and 1e6
  DoFs (n = round((N^(1/3) - 1) / p), the sweep's sizing rule): the iteration
  counts equal the oracle's (deal.II SolverCG + ReductionControl semantics).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def mf():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import benchmarks_gb300 as mf
    mf.lib()
    return mf


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def host_bytes():
    return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")


def apply_gpu(mf, A, src, arith):
    import torch
    y = A.initialize_dof_vector()
    A.vmult(y, torch.from_numpy(src).cuda(), arith=arith)
    mf.check_device_errors()
    return y.cpu().numpy()


@pytest.fixture(scope="module")
def bench_case(mf, orc):
    ref = orc.BoxProblem(128, 128, 64, 4, amplitude=0.05)
    src = np.random.default_rng(1).uniform(-1, 1, ref.n_dofs)
    return ref, src, ref.apply(src)


@pytest.mark.parametrize("arith", ["df", "fp64"])
def test_bench_workload_matches_oracle(mf, bench_case, arith):
    ref, src, want = bench_case
    A = mf.LaplaceOperator(mf.BoxMesh(128, 128, 64, degree=4, amplitude=0.05))
    assert A.m() == ref.n_dofs == 67_634_433
    got = apply_gpu(mf, A, src, arith)
    assert rel(got, want) <= TOL
    np.testing.assert_array_equal(got[ref.constrained], src[ref.constrained])


@pytest.mark.parametrize("p,n", [(1, 530), (8, 66)])
def test_largest_sweep_meshes_match_oracle(mf, orc, p, n):
    n_cells = n ** 3
    need = n_cells * (p + 1) ** 3 * (6 * 8 + 4) + 6 * 8 * (p * n + 1) ** 3
    if host_bytes() < 2 * need:
        pytest.skip(f"host memory below {2 * need / 2**30:.0f} GiB for the oracle")
    ref = orc.BoxProblem(n, n, n, p, amplitude=0.05)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    want = ref.apply(src)
    del ref.G
    A = mf.LaplaceOperator(mf.BoxMesh(n, n, n, degree=p, amplitude=0.05))
    assert A.m() == (p * n + 1) ** 3
    for arith in ("df", "fp64"):
        assert rel(apply_gpu(mf, A, src, arith), want) <= TOL


def sweep_cells(p, target):
    return max(2, round((target ** (1.0 / 3.0) - 1) / p))


@pytest.mark.parametrize("target", [1e5, 1e6])
@pytest.mark.parametrize("p", range(1, 9))
def test_jacobi_cg_counts_match_oracle(mf, orc, p, target):
    n = sweep_cells(p, target)
    ref = orc.BoxProblem(n, n, n, p, amplitude=0.05)
    b_h = ref.rhs(7)
    _, info = ref.cg(b_h, diag_inv=orc.invert_diagonal(ref.diagonal()), reduce=1e-10,
                     max_steps=100000)
    A = mf.LaplaceOperator(mf.BoxMesh(n, n, n, degree=p, amplitude=0.05))
    b = A.rhs_uniform(7)
    P = A.get_matrix_diagonal_inverse()
    for arith in ("fp64", "df"):
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(100000, 1e-300, 1e-10)
        mf.SolverCG(ctl).solve(A, x, b, P, arith=arith)
        assert ctl.last_step() == info["steps"], (arith, ctl.last_step(), info["steps"])
