"""Multigrid preconditioner on the GPU against the CPU multigrid oracle.

Tolerances: FP32 operator apply 1e-5 relative; FP64 V-cycle 1e-9 relative
(the library's coarse Jacobi-CG stops at 1e-12, the oracle solves the coarse
problem exactly); FP32 V-cycle 1e-4 relative; MG-CG solutions in FP32 and FP64
V-cycles agree to 1e-9.
"""
import ctypes

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


@pytest.fixture(scope="module")
def mgo():
    from oracle import mg_oracle
    return mg_oracle.MGOracle(8, 8, 4, 4, amplitude=0.1)


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("p", [1, 3, 4, 6])
def test_fp32_operator(mf, orc, p):
    import torch
    from benchmarks_gb300 import _abi
    A = mf.LaplaceOperator(mf.BoxMesh(4, 3, 5, degree=p, amplitude=0.1))
    ref = orc.BoxProblem(4, 3, 5, p, amplitude=0.1)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    s32 = torch.from_numpy(src.astype(np.float32)).cuda()
    d32 = torch.zeros_like(s32)
    _abi.check(mf.lib().mfgb_vmult_f32(A.handle, ctypes.c_void_p(d32.data_ptr()),
                                       ctypes.c_void_p(s32.data_ptr()), mf._stream_ptr()))
    assert rel(d32.cpu().numpy().astype(np.float64), ref.apply(src)) <= 1e-5


def test_hierarchy_matches_oracle(mf, mgo):
    M = mf.MGPreconditioner(mf.BoxMesh(8, 8, 4, degree=4, amplitude=0.1), precision=64)
    assert [l["degree"] for l in M.levels] == [L.degree for L in mgo.levels] == [4, 2, 1, 1]
    assert [l["dofs"] for l in M.levels] == [L.n for L in mgo.levels]
    for l, L in zip(M.levels[:-1], mgo.levels[:-1]):
        assert l["lambda_max"] == pytest.approx(L.lmax, rel=1e-10)


@pytest.mark.parametrize("precision,tol", [(64, 1e-9), (32, 1e-4)])
def test_vcycle_matches_oracle(mf, mgo, precision, tol):
    import torch
    mesh = mf.BoxMesh(8, 8, 4, degree=4, amplitude=0.1)
    M = mf.MGPreconditioner(mesh, precision=precision)
    A = mf.LaplaceOperator(mesh)
    r = A.rhs_uniform(5)
    z = A.initialize_dof_vector()
    M.vmult(z, r)
    want = mgo.vcycle(r.cpu().numpy())
    assert rel(z.cpu().numpy(), want) <= tol
    # the V-cycle is a linear, symmetric operator (up to rounding)
    r2 = A.rhs_uniform(6)
    z2 = A.initialize_dof_vector()
    M.vmult(z2, r2)
    a, b = float(torch.dot(r2, z)), float(torch.dot(r, z2))
    assert abs(a - b) <= (1e-9 if precision == 64 else 1e-4) * abs(a)


def test_mg_cg_matches_oracle_and_mixed_precision(mf, orc, mgo):
    import torch
    mesh = mf.BoxMesh(8, 8, 4, degree=4, amplitude=0.1)
    A = mf.LaplaceOperator(mesh)
    b = A.rhs_uniform(11)
    x_orc, info = mgo.pcg(b.cpu().numpy(), reduce=1e-10)
    sols = {}
    for prec in (64, 32):
        M = mf.MGPreconditioner(mesh, precision=prec)
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(200, 1e-300, 1e-10)
        mf.SolverCG(ctl).solve(A, x, b, M)
        assert ctl.last_value() <= 1e-10 * ctl.initial_value()
        assert ctl.last_step() <= 25
        if prec == 64:
            assert abs(ctl.last_step() - info["steps"]) <= 1
        sols[prec] = x.cpu().numpy()
    assert rel(sols[64], x_orc) <= 1e-9
    assert rel(sols[32], sols[64]) <= 1e-9
    # far fewer iterations than Jacobi-CG on the same problem
    ctl = mf.ReductionControl(100000, 1e-300, 1e-10)
    x = A.initialize_dof_vector()
    mf.SolverCG(ctl).solve(A, x, b, A.get_matrix_diagonal_inverse())
    assert ctl.last_step() > 3 * 25


def test_odd_mesh_hierarchy_and_vcycle(mf):
    """Cell counts that are not powers of two coarsen too (level l keeps the
    fine nodes min(k 2^l, n)); hierarchy, lambda_max and the FP64 V-cycle
    match the oracle."""
    from oracle import mg_oracle
    mgo = mg_oracle.MGOracle(7, 7, 5, 2, amplitude=0.08, coarse_cells=2)
    mesh = mf.BoxMesh(7, 7, 5, degree=2, amplitude=0.08)
    M = mf.MGPreconditioner(mesh, precision=64, coarse_cells=2)
    assert [l["dofs"] for l in M.levels] == [L.n for L in mgo.levels]
    assert [l["degree"] for l in M.levels] == [2, 1, 1, 1]
    for l, L in zip(M.levels[:-1], mgo.levels[:-1]):
        assert l["lambda_max"] == pytest.approx(L.lmax, rel=1e-10)
    A = mf.LaplaceOperator(mesh)
    r = A.rhs_uniform(3)
    z = A.initialize_dof_vector()
    M.vmult(z, r)
    assert rel(z.cpu().numpy(), mgo.vcycle(r.cpu().numpy())) <= 1e-9
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(200, 1e-300, 1e-10)
    mf.SolverCG(ctl).solve(A, x, r, M)
    _, info = mgo.pcg(r.cpu().numpy(), reduce=1e-10)
    assert abs(ctl.last_step() - info["steps"]) <= 1 and ctl.last_step() <= 30


@pytest.mark.parametrize("n", [19, 25, 31])
def test_odd_mesh_mg_cg_converges_fast(mf, n):
    """Odd cell counts that used to leave a coarse problem too large for the
    dense coarse solve now reach the 4^3 coarse mesh."""
    mesh = mf.BoxMesh(n, n, n, degree=2, amplitude=0.05)
    M = mf.MGPreconditioner(mesh, precision=32)
    assert M.levels[-1]["dofs"] <= 5 ** 3
    A = mf.LaplaceOperator(mesh)
    b = A.rhs_uniform(n)
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(200, 1e-300, 1e-10)
    mf.SolverCG(ctl).solve(A, x, b, M)
    assert ctl.last_value() <= 1e-10 * ctl.initial_value()
    assert ctl.last_step() <= 25


def test_shared_fine_operator(mf):
    """mfgb_mg_setup_shared: the finest level borrows the caller's operator; the
    hierarchy, the V-cycle and the solve match the stand-alone set-up."""
    mesh = mf.BoxMesh(8, 8, 4, degree=4, amplitude=0.1)
    A = mf.LaplaceOperator(mesh)
    M0 = mf.MGPreconditioner(mesh, precision=32)
    M1 = mf.MGPreconditioner(mesh, precision=32, operator=A)
    assert [l["dofs"] for l in M0.levels] == [l["dofs"] for l in M1.levels]
    for a, b in zip(M0.levels, M1.levels):
        assert a["lambda_max"] == pytest.approx(b["lambda_max"], rel=1e-6)
    r = A.rhs_uniform(9)
    z0, z1 = A.initialize_dof_vector(), A.initialize_dof_vector()
    M0.vmult(z0, r)
    M1.vmult(z1, r)
    assert rel(z1.cpu().numpy(), z0.cpu().numpy()) <= 1e-5
    its = []
    for M in (M0, M1):
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(200, 1e-300, 1e-10)
        mf.SolverCG(ctl).solve(A, x, r, M)
        its.append(ctl.last_step())
    assert its[0] == its[1]
    del M1
    y = A.initialize_dof_vector()
    A.vmult(y, r)  # the operator survives the hierarchy
    with pytest.raises(ValueError):
        mf.MGPreconditioner(mf.BoxMesh(8, 8, 2, degree=4), operator=A)
