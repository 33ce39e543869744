"""The bulk-TMA kernels on meshes with several batches per CTA, so that the
pipelined path runs: the next batch's G and dof-map tiles copied while the
current batch computes, and the next gather prefetched into registers.  The
small meshes of the other tests give every CTA at most one batch.  Collocation
(every TMA shape), Gauss-point, Helmholtz, BP3 and BK6 forms against the oracle; 1e-12
relative for FP64 and double-float, 1e-5 for FP32."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# cells per direction: a few thousand cells, i.e. 1.1-4 batches per resident CTA
MESH = {2: (32, 32, 24), 4: (24, 24, 16), 5: (16, 16, 16), 7: (12, 12, 10)}


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


def with_shape(mf, arith, p, shape, fn):
    from benchmarks_gb300 import _abi, autotune
    L = mf.lib()
    a = autotune.ARITHS[arith]
    old = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(a, p, ctypes.byref(old)))
    try:
        _abi.check(L.mfgb_set_kernel_shape(a, p, shape))
        return fn()
    finally:
        _abi.check(L.mfgb_set_kernel_shape(a, p, old.value))


@pytest.mark.parametrize("shape", [2, 4])
@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_collocation_tma_pipelined(mf, orc, p, arith, shape):
    import torch
    cells = MESH[p]
    ref = orc.BoxProblem(*cells, p, amplitude=0.06)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)

    def run():
        A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06))
        y = A.initialize_dof_vector()
        A.vmult(y, torch.from_numpy(src).cuda(), arith=arith)
        return y.cpu().numpy()

    y = with_shape(mf, arith, p, shape, run)
    from benchmarks_gb300 import _abi
    _abi.check(mf.lib().mfgb_check_device_errors(None))
    assert rel(y, ref.apply(src)) <= 1e-12


@pytest.mark.parametrize("shape", [2, 4])
@pytest.mark.parametrize("p", [2, 4, 5])
def test_collocation_tma_pipelined_fp32(mf, orc, p, shape):
    import torch
    from benchmarks_gb300 import _abi
    cells = MESH[p]
    ref = orc.BoxProblem(*cells, p, amplitude=0.06)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    L = mf.lib()

    def run():
        A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06))
        s32 = torch.from_numpy(src.astype(np.float32)).cuda()
        d32 = torch.zeros_like(s32)
        _abi.check(L.mfgb_vmult_f32(A.handle, ctypes.c_void_p(d32.data_ptr()),
                                    ctypes.c_void_p(s32.data_ptr()), mf._stream_ptr()))
        return d32.cpu().numpy().astype(np.float64)

    y = with_shape(mf, "fp32", p, shape, run)
    _abi.check(L.mfgb_check_device_errors(None))
    assert rel(y, ref.apply(src)) <= 1e-5


@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_gauss_tma_pipelined(mf, orc, p, arith):
    import torch
    from benchmarks_gb300 import _abi
    cells = MESH[p]
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06), quadrature="gauss")
    ref = orc.GaussProblem(*cells, p, amplitude=0.06)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, torch.from_numpy(src).cuda(), arith=arith)
    _abi.check(mf.lib().mfgb_check_device_errors(None))
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12


@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_helmholtz_tma_pipelined(mf, orc, p, arith):
    import torch
    from benchmarks_gb300 import _abi
    cells = MESH[p]
    H = mf.HelmholtzOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06), arith=arith)
    ref = orc.HelmholtzProblem(*cells, p, amplitude=0.06)
    src = np.random.default_rng(5).uniform(-1, 1, ref.n_dofs)
    dst = H.initialize_dof_vector()
    H.vmult(dst, torch.from_numpy(src).cuda())
    _abi.check(mf.lib().mfgb_check_device_errors(None))
    assert rel(dst.cpu().numpy(), ref.apply(src)) <= 1e-12


@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_bp3_tma_pipelined(mf, orc, p, arith):
    import torch
    from benchmarks_gb300 import _abi
    cells = MESH[p]
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06), arith=arith,
                           quadrature="bp3")
    ref = orc.GaussProblem(*cells, p, nq=p + 2, amplitude=0.06)
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, torch.from_numpy(src).cuda())
    _abi.check(mf.lib().mfgb_check_device_errors(None))
    assert rel(y.cpu().numpy(), ref.apply(src)) <= 1e-12


@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("p", [2, 4, 7])
def test_bk6_tma_pipelined(mf, orc, p, arith):
    """BK6 (3 interleaved components): each component through the scalar
    operator, with the component gathers prefetched across batches."""
    import torch
    from benchmarks_gb300 import _abi
    cells = MESH[p]
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.06))
    ref = orc.BoxProblem(*cells, p, amplitude=0.06)
    src = np.random.default_rng(p + 20).uniform(-1, 1, 3 * ref.n_dofs)
    y = torch.zeros(3 * ref.n_dofs, dtype=torch.float64, device="cuda")
    A.vmult_vector(y, torch.from_numpy(src).cuda(), arith=arith)
    _abi.check(mf.lib().mfgb_check_device_errors(None))
    want = np.empty_like(src)
    for c in range(3):
        want[c::3] = ref.apply(src[c::3])
    assert rel(y.cpu().numpy(), want) <= 1e-12
