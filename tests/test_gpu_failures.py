"""Failure paths, made on the host or by a wait that runs out (nothing faults,
traps or hangs the GPU).  The reference exits on any error
(CEED_BK/src/BK5/templated_cuda_benchmark.cc:9-27); the library returns statuses.

* Bounded copy waits: the test hook arms the offset-accumulation kernel's first
  geometric-factor wait without issuing the copy and lowers the limit to 1 ms;
  the wait runs out with nothing in flight, mfgb_check_device_errors reports
  MFGB_ERR_TIMEOUT (a solver returns it), and the next application is correct.
* Allocation failure: the n-th device allocation fails on the host; every call
  returns MFGB_ERR_OUT_OF_MEMORY and frees what it had allocated.
* Determinism of the atomic scatter: repeated applications agree to a few ulps
  and conjugate gradients keep their iteration count run to run at 1e7 DoFs.
"""
import gc

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


def test_copy_wait_timeout_is_reported_and_recovers(mf, orc):
    import torch
    from benchmarks_gb300 import MfgbError, _abi
    L = mf.lib()
    A = mf.LaplaceOperator(mf.BoxMesh(6, 5, 5, degree=4, amplitude=0.05))
    ref = orc.BoxProblem(6, 5, 5, 4, amplitude=0.05)
    src = np.random.default_rng(3).uniform(-1, 1, ref.n_dofs)
    u = torch.from_numpy(src).cuda()
    y = A.initialize_dof_vector()
    A.vmult(y, u, arith="df")  # builds the scaled pairs, loads the kernel
    mf.check_device_errors()
    _abi.check(L.mfgb_test_expire_copy_wait(1))
    A.vmult(y, u, arith="df")
    with pytest.raises(MfgbError) as e:
        mf.check_device_errors()
    assert e.value.status == _abi.ERR_TIMEOUT
    mf.check_device_errors()  # cleared by the read
    A.vmult(y, u, arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12
    # inside a solve: conjugate gradients return the status, and the next solve works
    b = A.rhs_uniform(1)
    x = A.initialize_dof_vector()
    _abi.check(L.mfgb_test_expire_copy_wait(1))
    ctl = mf.ReductionControl(1000, 1e-300, 1e-8)
    with pytest.raises(MfgbError) as e:
        mf.SolverCG(ctl).solve(A, x, b, A.get_matrix_diagonal_inverse(), arith="df")
    assert e.value.status == _abi.ERR_TIMEOUT
    x.zero_()
    mf.SolverCG(ctl).solve(A, x, b, A.get_matrix_diagonal_inverse(), arith="df")
    _, info = ref.cg(b.cpu().numpy(), diag_inv=orc.invert_diagonal(ref.diagonal()), reduce=1e-8,
                     max_steps=1000)
    assert ctl.last_step() == info["steps"]


def test_allocation_failure_frees_and_reports(mf):
    import torch
    from benchmarks_gb300 import MfgbError, _abi
    L = mf.lib()
    mesh = mf.BoxMesh(8, 8, 6, degree=3, amplitude=0.05)
    A0 = mf.LaplaceOperator(mesh)  # kernels loaded, caches warm
    y0 = A0.initialize_dof_vector()
    A0.vmult(y0, A0.rhs_uniform(1), arith="df")
    M0 = mf.MGPreconditioner(mesh, precision=32, operator=A0)
    del M0

    def attempt():
        A = mf.LaplaceOperator(mesh)
        y = A.initialize_dof_vector()
        A.vmult(y, A.rhs_uniform(2), arith="df")
        M = mf.MGPreconditioner(mesh, precision=32, operator=A)
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(100, 1e-300, 1e-6)
        mf.SolverCG(ctl).solve(A, x, y, M)

    failed = 0
    try:
        for n in range(1, 40):
            gc.collect()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            free0 = torch.cuda.mem_get_info()[0]
            _abi.check(L.mfgb_test_fail_allocation(n))
            try:
                attempt()
            except MfgbError as e:
                assert e.status == _abi.ERR_OUT_OF_MEMORY, (n, e)
                failed += 1
            finally:
                _abi.check(L.mfgb_test_fail_allocation(0))
            gc.collect()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            assert torch.cuda.mem_get_info()[0] >= free0 - (2 << 20), n  # nothing leaked
    finally:
        _abi.check(L.mfgb_test_fail_allocation(0))
    assert failed >= 10  # the hook reached allocations in the operator, MG set-up and CG


def test_scatter_is_reproducible_run_to_run(mf):
    """Atomic FP64 scatter: results may differ in the last bits between runs,
    like the reference's Kokkos atomic_add (bakeoff_problems_dealii/include/
    bk3_kokkos_kernel.h:424); the spread stays at the rounding level and the
    Jacobi-CG iteration count at 1e7 DoFs does not change."""
    import torch
    A = mf.LaplaceOperator(mf.BoxMesh(54, 54, 54, degree=4, amplitude=0.05))
    assert A.m() > 1e7
    u = A.rhs_uniform(9)
    ys = []
    for _ in range(5):
        y = A.initialize_dof_vector()
        A.vmult(y, u)
        ys.append(y)
    for y in ys[1:]:
        assert float(torch.linalg.norm(y - ys[0]) / torch.linalg.norm(ys[0])) <= 1e-15
    P = A.get_matrix_diagonal_inverse()
    steps = []
    for _ in range(2):
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(100000, 1e-300, 1e-10)
        mf.SolverCG(ctl).solve(A, x, u, P)
        steps.append(ctl.last_step())
    assert steps[0] == steps[1]
