"""The Gauss-quadrature (BP5-variant) operator on the GPU: parity with the
oracle's Gauss form, and the reference's published CG iteration counts and
reductions reproduced on the GPU (cycles 8..10 of the reference's scaling
study; bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/results/
1_GPU.out:640-642).  Tolerance 1e-12 relative for the operator."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mf():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import benchmarks_gb300 as mf
    mf.lib()
    return mf


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("p", range(1, 9))
@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_gauss_operator_matches_oracle(mf, orc, p, arith):
    import torch
    cells = (3, 2, 3)
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.07), quadrature="gauss")
    ref = orc.GaussProblem(*cells, p, amplitude=0.07)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, torch.from_numpy(src).cuda(), arith=arith)
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12


@pytest.mark.parametrize("cycle", [8, 9, 10])
def test_published_cg_counts_on_gpu(mf, orc, cycle):
    import torch
    path = os.path.join(os.path.dirname(__file__), "golden", "published_bp5_cg.json")
    rows = {r["dofs"]: r for r in json.load(open(path))["rows"]}
    cells, lo, hi = orc.reference_scaling_mesh(cycle, 4)
    mesh = mf.BoxMesh(*cells, degree=4, amplitude=0.0, lo=lo, hi=hi)
    A = mf.LaplaceOperator(mesh, quadrature="gauss")
    pub = rows[A.m()]
    assert A.n_cells == pub["cells"]
    b = torch.from_numpy(orc.GaussProblem(*cells, 4, lo=lo, hi=hi).rhs_unit()).cuda()
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(1000000000 // 2, 1e-16, 1e-9)
    mf.SolverCG(ctl).solve(A, x, b)
    assert ctl.last_step() == pub["cg_its"]
    red = (ctl.last_value() / ctl.initial_value()) ** (1.0 / ctl.last_step())
    assert f"{red:.3e}" == f"{pub['cg_reduction']:.3e}"
