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


def torch_from(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


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


@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
def test_helmholtz_operator_matches_oracle(mf, orc, p, arith):
    """bp5_kokkos's Helmholtz operator (mass + stiffness at QGauss(p+1)) on a
    deformed box: vmult and the exact diagonal against the oracle."""
    cells = (3, 2, 4) if p <= 4 else (2, 2, 2)
    H = mf.HelmholtzOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.05), arith=arith)
    ref = orc.HelmholtzProblem(*cells, p, amplitude=0.05)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    dst = H.initialize_dof_vector()
    H.vmult(dst, torch_from(src))
    assert rel(dst.cpu().numpy(), ref.apply(src)) <= 1e-12
    d = H.compute_diagonal()
    assert rel(d.cpu().numpy(), ref.diagonal()) <= 1e-13


@pytest.mark.parametrize("p", [2, 4])
def test_gauss_diagonal_matches_oracle(mf, orc, p):
    A = mf.LaplaceOperator(mf.BoxMesh(3, 3, 2, degree=p, amplitude=0.08), quadrature="gauss")
    ref = orc.GaussProblem(3, 3, 2, p, amplitude=0.08)
    d = A.compute_diagonal()
    dr = np.zeros(ref.n_dofs)
    orc._gauss_sigs().orc_gauss_diagonal(ref.n, ref.nq, orc._p(ref.B), orc._p(ref.DG), ref.n_cells,
                                         orc._p(ref.map), orc._p(ref.Gg), None, ref.n_dofs,
                                         ref.constrained.size, orc._p(ref.constrained), orc._p(dr))
    assert rel(d.cpu().numpy(), dr) <= 1e-13


def test_helmholtz_jacobi_pcg_counts(mf, orc):
    """Jacobi-PCG with bp5_kokkos's ReductionControl(100, 1e-15, 1e-8): the same
    iteration count as the oracle and a solution within the tolerance."""
    mesh = mf.BoxMesh(4, 4, 3, degree=3, amplitude=0.05)
    H = mf.HelmholtzOperator(mesh)
    ref = orc.HelmholtzProblem(4, 4, 3, 3, amplitude=0.05)
    b = H.rhs_uniform(17)
    x = H.initialize_dof_vector()
    ctl = mf.ReductionControl(100, 1e-15, 1e-8)
    mf.SolverCG(ctl).solve(H, x, b, H.get_matrix_diagonal_inverse())
    dinv = 1.0 / ref.diagonal()
    xr, info = ref.cg(b.cpu().numpy(), diag_inv=dinv)
    assert ctl.last_step() == info["steps"]
    assert rel(x.cpu().numpy(), xr) <= 1e-9


@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("p", range(1, 9))
def test_bp3_operator_matches_oracle(mf, orc, p, arith):
    """BP3: the Laplacian at QGauss(p+2) (L-vector, gather/scatter through the
    dof map) on a deformed box, against the oracle's Gauss problem with
    nq = p + 2; the exact diagonal too."""
    cells = (3, 2, 3) if p <= 5 else (2, 2, 2)
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.07), arith=arith,
                           quadrature="bp3")
    ref = orc.GaussProblem(*cells, p, nq=p + 2, amplitude=0.07)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, torch_from(src))
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12
    if arith == "fp64":
        dr = np.zeros(ref.n_dofs)
        orc._gauss_sigs().orc_gauss_diagonal(ref.n, ref.nq, orc._p(ref.B), orc._p(ref.DG),
                                             ref.n_cells, orc._p(ref.map), orc._p(ref.Gg), None,
                                             ref.n_dofs, ref.constrained.size,
                                             orc._p(ref.constrained), orc._p(dr))
        assert rel(A.compute_diagonal().cpu().numpy(), dr) <= 1e-13


@pytest.mark.parametrize("p", [2, 4, 7])
def test_bp3_many_batches_match_oracle(mf, orc, p):
    """More cells than one wave of CTAs (every CTA runs several batches of the
    pipeline, the last one partial), double-float against the oracle."""
    cells = {2: (14, 12, 11), 4: (12, 11, 9), 7: (8, 7, 7)}[p]
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06), quadrature="bp3")
    ref = orc.GaussProblem(*cells, p, nq=p + 2, amplitude=0.06)
    src = np.random.default_rng(10 + p).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, torch_from(src), arith="df")
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12


def test_bp3_cg_counts_match_oracle(mf, orc):
    mesh = mf.BoxMesh(4, 3, 3, degree=3, amplitude=0.05)
    A = mf.LaplaceOperator(mesh, quadrature="bp3")
    ref = orc.GaussProblem(4, 3, 3, 3, nq=5, amplitude=0.05)
    b = A.rhs_uniform(4)
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(1000, 1e-300, 1e-10)
    mf.SolverCG(ctl).solve(A, x, b, A.get_matrix_diagonal_inverse())
    dinv = 1.0 / A.compute_diagonal().cpu().numpy()
    xr, info = ref.cg(b.cpu().numpy(), diag_inv=dinv, tol=1e-300, reduce=1e-10)
    assert ctl.last_step() == info["steps"]
    assert rel(x.cpu().numpy(), xr) <= 1e-9
