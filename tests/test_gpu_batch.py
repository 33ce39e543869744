"""Batched solves on the GPU against the same problems solved one by one
(single-problem operator, multigrid and CG) and against the CPU oracle.

Tolerances: batched operator 1e-13 relative per problem (same double-float
arithmetic, atomics in another order); batched FP32 V-cycle 1e-5 relative
(FP32 rounding; the coarse levels use an exact inverse instead of a Jacobi-CG
to 1e-12); CG iteration counts within one of the single-problem solves;
solutions 1e-9 relative."""
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
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


SPECS = [  # (nx, ny, nz, degree, amplitude): uneven degrees and sizes, odd counts
    (3, 3, 3, 2, 0.05), (4, 3, 5, 3, 0.08), (6, 6, 6, 4, 0.1), (2, 2, 2, 2, 0.0),
    (7, 5, 6, 5, 0.03), (5, 5, 5, 1, 0.07), (2, 2, 2, 1, 0.02), (9, 9, 9, 2, 0.09),
    (4, 4, 4, 7, 0.06), (3, 4, 3, 6, 0.04),
]


@pytest.fixture(scope="module")
def batch(mf):
    meshes = [mf.BoxMesh(*s[:3], degree=s[3], amplitude=s[4]) for s in SPECS]
    return meshes, mf.BatchSolver(meshes)


def test_layout(mf, batch):
    meshes, B = batch
    assert B.n_problems == len(meshes)
    assert list(np.diff(B.offsets)) == [m.n_dofs for m in meshes]
    for m, lv in zip(meshes, B.levels):
        assert lv == len(mf.MGPreconditioner(m, precision=32).levels)
    assert B.levels[6] == 1  # 2x2x2 Q1: the coarse solve is the whole V-cycle


def test_vmult_matches_single_problems(mf, batch):
    import torch
    meshes, B = batch
    src = torch.from_numpy(np.random.default_rng(3).uniform(-1, 1, B.n_dofs)).cuda()
    dst = B.initialize_dof_vector()
    B.vmult(dst, src)
    for m, s, d in zip(meshes, B.split(src), B.split(dst)):
        A = mf.LaplaceOperator(m)
        want = A.initialize_dof_vector()
        A.vmult(want, s.contiguous())
        assert rel(d.cpu().numpy(), want.cpu().numpy()) <= 1e-13


def test_vmult_matches_oracle(mf, orc, batch):
    import torch
    meshes, B = batch
    src = torch.from_numpy(np.random.default_rng(4).uniform(-1, 1, B.n_dofs)).cuda()
    dst = B.initialize_dof_vector()
    B.vmult(dst, src)
    for i in (0, 4, 8):
        m = meshes[i]
        ref = orc.BoxProblem(m.nx, m.ny, m.nz, m.degree, amplitude=m.amplitude)
        s = B.split(src)[i].cpu().numpy()
        assert rel(B.split(dst)[i].cpu().numpy(), ref.apply(s)) <= 1e-12


def test_precondition_matches_single_vcycles(mf, batch):
    meshes, B = batch
    seeds = list(range(100, 100 + B.n_problems))
    r = B.rhs_uniform(seeds)
    z = B.initialize_dof_vector()
    B.precondition(z, r)
    for i, (m, ri, zi) in enumerate(zip(meshes, B.split(r), B.split(z))):
        A = mf.LaplaceOperator(m)
        assert np.array_equal(ri.cpu().numpy(), A.rhs_uniform(seeds[i]).cpu().numpy())
        M = mf.MGPreconditioner(m, precision=32)
        want = A.initialize_dof_vector()
        M.vmult(want, ri.contiguous())
        assert rel(zi.cpu().numpy(), want.cpu().numpy()) <= 1e-5, i


def test_solve_matches_single_solves(mf, orc, batch):
    meshes, B = batch
    seeds = [7 * i + 1 for i in range(B.n_problems)]
    b = B.rhs_uniform(seeds)
    x = B.initialize_dof_vector()
    B.solve(x, b, max_steps=100, reduce=1e-10)
    for i, m in enumerate(meshes):
        info = B.infos[i]
        assert info["converged"] and info["last"] <= 1e-10 * info["initial"]
        A = mf.LaplaceOperator(m)
        M = mf.MGPreconditioner(m, precision=32)
        xi = A.initialize_dof_vector()
        ctl = mf.ReductionControl(100, 1e-300, 1e-10)
        mf.SolverCG(ctl).solve(A, xi, B.split(b)[i].contiguous(), M)
        assert abs(info["steps"] - ctl.last_step()) <= 1, (i, info, ctl.last_step())
        assert rel(B.split(x)[i].cpu().numpy(), xi.cpu().numpy()) <= 1e-9
    assert B.infos[6]["steps"] == 1  # exact coarse solve as the preconditioner
    assert B.replans >= 1  # converged problems were dropped from the launches
    # the residual of a solution, checked by the CPU oracle
    m = meshes[2]
    ref = orc.BoxProblem(m.nx, m.ny, m.nz, m.degree, amplitude=m.amplitude)
    xb, bb = B.split(x)[2].cpu().numpy(), B.split(b)[2].cpu().numpy()
    assert np.linalg.norm(bb - ref.apply(xb)) <= 2e-10 * np.linalg.norm(bb)


def test_not_converged_reports_every_problem(mf, batch):
    from benchmarks_gb300 import _abi
    meshes, B = batch
    b = B.rhs_uniform(list(range(B.n_problems)))
    x = B.initialize_dof_vector()
    with pytest.raises(_abi.MfgbError) as e:
        B.solve(x, b, max_steps=2, reduce=1e-14)
    assert e.value.status == _abi.ERR_NOT_CONVERGED
    assert all(i["steps"] <= 2 for i in B.infos)
    assert B.infos[6]["converged"]  # one step solves the single-level problem
    assert not B.infos[2]["converged"] and B.infos[2]["steps"] == 2

