"""Conjugate gradients on the GPU: iteration counts identical to the oracle's
(deal.II SolverCG + ReductionControl semantics)."""
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


@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("jacobi", [True, False])
def test_cg_bp5_cpu_config(mf, orc, arith, jacobi):
    """BP5 plain on the CPU config: 16^3 cells, p = 3, a = 0.05, Jacobi-CG to 1e-8."""
    import torch
    mesh = mf.BoxMesh(16, 16, 16, degree=3, amplitude=0.05)
    A = mf.LaplaceOperator(mesh, arith=arith)
    ref = orc.BoxProblem(16, 16, 16, 3, amplitude=0.05)
    b_h = ref.rhs(2025)
    dinv_h = orc.invert_diagonal(ref.diagonal()) if jacobi else None
    x_ref, info = ref.cg(b_h, diag_inv=dinv_h, reduce=1e-8, max_steps=10000)
    b = A.rhs_uniform(2025)
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(10000, 1e-300, 1e-8)
    P = A.get_matrix_diagonal_inverse() if jacobi else mf.PreconditionIdentity()
    mf.SolverCG(ctl).solve(A, x, b, P)
    assert ctl.last_step() == info["steps"]
    assert ctl.initial_value() == pytest.approx(info["initial"], rel=1e-14)
    assert ctl.last_value() <= 1e-8 * ctl.initial_value()
    xs = x.cpu().numpy()
    assert np.linalg.norm(xs - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
    r = b_h - ref.apply(xs)
    assert np.linalg.norm(r) <= 1.01e-8 * info["initial"]


def test_cg_not_converged_and_trivial(mf):
    import torch
    from benchmarks_gb300 import MfgbError
    A = mf.LaplaceOperator(mf.BoxMesh(4, 4, 4, degree=2))
    b = A.rhs_uniform(1)
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(5, 1e-300, 1e-12)
    with pytest.raises(MfgbError) as e:
        mf.SolverCG(ctl).solve(A, x, b)
    assert e.value.status == 3 and ctl.last_step() == 5
    # zero right-hand side: converged before the first step
    z = A.initialize_dof_vector()
    x.zero_()
    ctl = mf.ReductionControl(100, 1e-300, 1e-8)
    mf.SolverCG(ctl).solve(A, x, z)
    assert ctl.last_step() == 0 and float(x.abs().max()) == 0.0


def test_dot_deterministic(mf):
    import torch
    g = torch.Generator(device="cuda").manual_seed(0)
    a = torch.rand(10_000_019, dtype=torch.float64, device="cuda", generator=g)
    b = torch.rand(10_000_019, dtype=torch.float64, device="cuda", generator=g)
    d1, d2 = mf.dot(a, b), mf.dot(a, b)
    assert d1 == d2
    assert d1 == pytest.approx(float(torch.dot(a, b)), rel=1e-13)
