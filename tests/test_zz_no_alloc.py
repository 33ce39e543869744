"""The allocation-free conjugate-gradient entry point.

mfgb_cg_solve_noalloc serves callers that cannot allocate device memory while
they solve (their own allocator owns the device, or the solve runs inside
another code's time loop).  Its scratch is a fixed device array shared by all
calls, so this test checks it against mfgb_cg_solve (which allocates its own
work vectors) on two calls in a row: the second call starts from whatever the
first one left in the scratch.  Tolerance: same iteration count and the
solution within 1e-7 relative, the tolerance the solver tests use for CG
solutions (tests/test_gpu_cg.py).
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


def _solve(mf, entry, A, b, inv_diag, arith, reduce=1e-10):
    from benchmarks_gb300 import _abi
    x = A.initialize_dof_vector()
    ctl = _abi.CgControl(100000, 1e-300, reduce, mf._arith(arith))
    info = _abi.SolveInfo()
    inv = ctypes.c_void_p(inv_diag.data_ptr()) if inv_diag is not None else None
    st = getattr(mf.lib(), entry)(A.handle, ctypes.c_void_p(b.data_ptr()),
                                  ctypes.c_void_p(x.data_ptr()), inv, ctypes.byref(ctl),
                                  ctypes.byref(info), mf._stream_ptr())
    _abi.check(st)
    return x.cpu().numpy(), info.steps, info.last


@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_noalloc_cg_matches_allocating_cg(mf, arith):
    A = mf.LaplaceOperator(mf.BoxMesh(12, 10, 9, degree=3, amplitude=0.05))
    inv = A.get_matrix_diagonal_inverse().get_vector()
    for seed in (1, 2):  # two calls in a row on the shared scratch
        b = A.rhs_uniform(seed)
        x_ref, steps_ref, last_ref = _solve(mf, "mfgb_cg_solve", A, b, inv, arith)
        x, steps, last = _solve(mf, "mfgb_cg_solve_noalloc", A, b, inv, arith)
        assert steps == steps_ref
        assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)
        assert last == pytest.approx(last_ref, rel=1e-6)
    # identity preconditioner as well
    b = A.rhs_uniform(3)
    x_ref, steps_ref, _ = _solve(mf, "mfgb_cg_solve", A, b, None, arith)
    x, steps, _ = _solve(mf, "mfgb_cg_solve_noalloc", A, b, None, arith)
    assert steps == steps_ref
    assert np.linalg.norm(x - x_ref) <= 1e-7 * np.linalg.norm(x_ref)


@pytest.mark.parametrize("arith", ["df", "fp64"])
def test_noalloc_cg_first_on_a_fresh_operator(mf, orc, arith):
    """No allocating call has built the operator's double-float copy of G, so a
    double-float solve splits the FP64 factors on load.  Checked against the
    oracle's CG (same iteration count, solution to 1e-7), on two calls in a
    row; the second call leaves the device's free memory unchanged (the first
    may still load kernels)."""
    import torch
    mesh = mf.BoxMesh(9, 8, 7, degree=3, amplitude=0.05)
    ref = orc.BoxProblem(9, 8, 7, 3, amplitude=0.05)
    A = mf.LaplaceOperator(mesh)  # geometry only: no split copy of G yet
    inv_h = orc.invert_diagonal(ref.diagonal())
    inv = torch.from_numpy(inv_h).cuda()
    from benchmarks_gb300 import _abi
    for k, seed in enumerate((4, 5)):
        b = A.rhs_uniform(seed)
        x_ref, info = ref.cg(b.cpu().numpy(), diag_inv=inv_h, reduce=1e-10, max_steps=100000)
        x = A.initialize_dof_vector()
        ctl = _abi.CgControl(100000, 1e-300, 1e-10, mf._arith(arith))
        sinfo = _abi.SolveInfo()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        _abi.check(mf.lib().mfgb_cg_solve_noalloc(
            A.handle, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
            ctypes.c_void_p(inv.data_ptr()), ctypes.byref(ctl), ctypes.byref(sinfo),
            mf._stream_ptr()))
        torch.cuda.synchronize()
        if k == 1:
            assert torch.cuda.mem_get_info()[0] == free0
        assert sinfo.steps == info["steps"]
        xs = x.cpu().numpy()
        assert np.linalg.norm(xs - x_ref) <= 1e-7 * np.linalg.norm(x_ref)


def test_noalloc_cg_rejects_too_large(mf):
    from benchmarks_gb300 import MfgbError
    A = mf.LaplaceOperator(mf.BoxMesh(26, 26, 26, degree=4))
    assert A.m() > 1048576
    b = A.rhs_uniform(1)
    with pytest.raises(MfgbError) as e:
        _solve(mf, "mfgb_cg_solve_noalloc", A, b, None, "fp64")
    assert e.value.status == 7 and "exceed" in str(e.value)
