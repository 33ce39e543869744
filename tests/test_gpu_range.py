"""Range of the FP64-accurate double-float arithmetic (MFGB_ARITH_FP64_DF).

* GLL collocation (BK5, and BK6 per component), the Gauss p+1 Laplacian and its
  Helmholtz form, and BP3 scale every cell by a power of two: source vectors and
  geometric factors scaled by 2^-100, 1e-30, 1e30 and 2^300 give the scaled
  oracle result to the operator's 1e-12 bar.
* The double-float kernels without per-cell scaling (the TwoSum collocation
  shapes 0-4, a seam given an unaligned G) take inputs whose largest magnitude
  lies in [2^-40, 2^55]:
  inside it they meet 1e-12, outside it they report MFGB_ERR_RANGE (the seam on
  the call, an operator application through the device error word).
* A NaN in the right-hand side ends conjugate gradients with MFGB_ERR_NONFINITE.
"""
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
    """|a - b| / |b|, both divided by max|b| first: the squares inside the norms
    of vectors near 1e-280 would underflow to zero"""
    m = float(np.max(np.abs(b)))
    if m == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.linalg.norm((a - b) / m) / np.linalg.norm(b / m))


def cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def box(orc):
    ref = orc.BoxProblem(4, 3, 3, 4, amplitude=0.1)
    src = np.random.default_rng(11).uniform(-1, 1, ref.n_dofs)
    return ref, src, ref.apply(src)


@pytest.mark.parametrize("scale", [2.0 ** -100, 1e-30, 1e30, 2.0 ** 300])
def test_gll_df_carries_any_source_scale(mf, box, scale):
    ref, src, want = box
    A = mf.LaplaceOperator(mf.BoxMesh(4, 3, 3, degree=4, amplitude=0.1))
    y = A.initialize_dof_vector()
    A.vmult(y, cuda(src * scale), arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), want * scale) <= TOL


@pytest.mark.parametrize("scale", [2.0 ** -100, 1e-30, 1e30, 2.0 ** 300, 1e-280])
def test_bp3_df_carries_any_source_scale(mf, orc, scale):
    """The BP3 operator (QGauss(p+2)) scales every cell like the collocation
    kernels: any source range meets the 1e-12 bar, exact zeros included."""
    ref = orc.GaussProblem(3, 3, 2, 3, nq=5, amplitude=0.05)
    A = mf.LaplaceOperator(mf.BoxMesh(3, 3, 2, degree=3, amplitude=0.05), quadrature="bp3")
    src = np.random.default_rng(6).uniform(-1, 1, ref.n_dofs)
    src[::7] = 0.0
    y = A.initialize_dof_vector()
    A.vmult(y, cuda(src * scale), arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), ref.apply(src) * scale) <= TOL


@pytest.mark.parametrize("scale", [1e-280, 2.0 ** -960])
def test_gll_df_tiny_cells_keep_exact_zeros(mf, box, scale):
    """Every cell's values below 2^-897: the cell scale offset is below -896, and
    source entries that are exactly zero must convert to zero."""
    ref, src, _ = box
    s = src.copy()
    s[::5] = 0.0
    A = mf.LaplaceOperator(mf.BoxMesh(4, 3, 3, degree=4, amplitude=0.1))
    y = A.initialize_dof_vector()
    A.vmult(y, cuda(s * scale), arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), ref.apply(s) * scale) <= TOL


@pytest.mark.parametrize("gscale", [2.0 ** -100, 1e-30, 1e30])
def test_gll_df_carries_any_geometry_scale(mf, box, gscale):
    ref, src, want = box
    A = mf.LaplaceOperator(degree=4, n_dofs=ref.n_dofs, dof_map=ref.map, G=ref.G * gscale,
                           constrained=ref.constrained)
    y = A.initialize_dof_vector()
    for sscale in (1.0, 1e-30):
        A.vmult(y, cuda(src * sscale), arith="df")
        mf.check_device_errors()
        want_s = want * gscale * sscale
        want_s[ref.constrained] = src[ref.constrained] * sscale  # identity rows are not scaled by G
        assert rel(y.cpu().numpy(), want_s) <= TOL


def test_twosum_shape_df_range_window(mf, box):
    """The TwoSum collocation kernels (shapes 0-4, chosen by
    mfgb_set_kernel_shape) carry no per-cell scaling: inside the window 1e-12,
    outside it the device range word reports MFGB_ERR_RANGE; the scaled
    default kernel has no window."""
    import ctypes
    from benchmarks_gb300 import MfgbError, _abi
    ref, src, want = box
    L = mf.lib()
    old = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(1, 4, ctypes.byref(old)))
    A = mf.LaplaceOperator(mf.BoxMesh(4, 3, 3, degree=4, amplitude=0.1))
    y = A.initialize_dof_vector()
    try:
        _abi.check(L.mfgb_set_kernel_shape(1, 4, 4))  # double-float, p = 4: TwoSum bulk-TMA
        for scale in (2.0 ** -30, 2.0 ** 40):  # inside the window
            A.vmult(y, cuda(src * scale), arith="df")
            mf.check_device_errors()
            assert rel(y.cpu().numpy(), want * scale) <= TOL
        for scale in (2.0 ** -100, 1e-30, 2.0 ** 300):  # outside: reported, not silent
            A.vmult(y, cuda(src * scale), arith="df")
            with pytest.raises(MfgbError) as e:
                mf.check_device_errors()
            assert e.value.status == _abi.ERR_RANGE
        mf.check_device_errors()  # the word was cleared
    finally:
        _abi.check(L.mfgb_set_kernel_shape(1, 4, old.value))
    A.vmult(y, cuda(src * 1e-30), arith="df")  # the scaled default kernel
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), want * 1e-30) <= TOL


@pytest.mark.parametrize("scale", [2.0 ** -100, 1e-30, 2.0 ** 300, 1e-280])
def test_helmholtz_df_carries_any_source_scale(mf, orc, scale):
    """The Helmholtz form (mass + stiffness at QGauss(p+1)) runs the scaled
    offset-accumulation kernel with JxW on each cell's G scale: any source
    scale meets the bar, as native FP64 does."""
    ref = orc.HelmholtzProblem(3, 3, 2, 3, amplitude=0.05)
    H = mf.HelmholtzOperator(mf.BoxMesh(3, 3, 2, degree=3, amplitude=0.05))
    src = np.random.default_rng(5).uniform(-1, 1, ref.n_dofs)
    want = ref.apply(src) * scale
    y = H.initialize_dof_vector()
    for arith in ("df", "fp64"):
        H.vmult(y, cuda(src * scale), arith=arith)
        mf.check_device_errors()
        assert rel(y.cpu().numpy(), want) <= TOL


@pytest.mark.parametrize("side", [2.0 ** -30, 2.0 ** 30])
def test_helmholtz_df_carries_any_domain_scale(mf, orc, side):
    """A box of side L scales G by L and JxW by L^3: the per-cell offset
    covers both, and the mass and stiffness terms, 2^120 apart in relative
    size across these cases, meet the bar together."""
    hi = (side, side, side)
    ref = orc.HelmholtzProblem(3, 3, 2, 3, amplitude=0.0, hi=hi)
    H = mf.HelmholtzOperator(mf.BoxMesh(3, 3, 2, degree=3, amplitude=0.0, hi=hi))
    src = np.random.default_rng(6).uniform(-1, 1, ref.n_dofs)
    y = H.initialize_dof_vector()
    H.vmult(y, cuda(src), arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), ref.apply(src)) <= TOL


@pytest.mark.parametrize("scale", [2.0 ** -100, 1e-30, 2.0 ** 300])
def test_gauss_df_carries_any_source_scale(mf, orc, scale):
    """The Gauss p+1 Laplacian runs the scaled offset-accumulation kernel:
    any source range meets the 1e-12 bar."""
    ref = orc.GaussProblem(3, 3, 2, 3, amplitude=0.05)
    A = mf.LaplaceOperator(mf.BoxMesh(3, 3, 2, degree=3, amplitude=0.05), quadrature="gauss")
    src = np.random.default_rng(5).uniform(-1, 1, ref.n_dofs)
    y = A.initialize_dof_vector()
    A.vmult(y, cuda(src * scale), arith="df")
    mf.check_device_errors()
    assert rel(y.cpu().numpy(), ref.apply(src) * scale) <= TOL


@pytest.mark.parametrize("scale", [(1e-30, 1.0), (1.0, 2.0 ** 100), (1e30, 1e-280)])
def test_evector_seam_df_carries_any_scale(mf, orc, scale):
    """The BK5 E-vector seam scales every element's G and input by powers of
    two inside the kernel: any FP64 range meets 1e-12."""
    import torch
    gs, us = scale
    p, nelmt = 3, 23
    nq = p + 1
    rng = np.random.default_rng(2)
    x, _ = orc.gll(nq)
    D = orc.derivative_matrix(x).reshape(-1)
    G = rng.uniform(0.1, 1, nelmt * 6 * nq ** 3)
    u = rng.uniform(-1, 1, nelmt * nq ** 3)
    out = torch.zeros(nelmt * nq ** 3, dtype=torch.float64, device="cuda")
    mf.bk5_evector(p, cuda(D), cuda(G * gs), cuda(u * us), out, arith="df")
    assert rel(out.cpu().numpy(), orc.evector(nq, D, G, u) * gs * us) <= TOL


def test_lvector_seam_df_scale_and_range(mf, orc):
    """The L-vector seam with a 16-byte aligned G scales every cell inside the
    kernel (any range); with an unaligned G it runs the TwoSum kernel, whose
    window the call checks: inside it 1e-12, outside it MFGB_ERR_RANGE."""
    from benchmarks_gb300 import MfgbError, _abi
    import torch
    ref = orc.BoxProblem(3, 3, 2, 3, amplitude=0.1)
    src = np.random.default_rng(9).uniform(-1, 1, ref.n_dofs)
    dmap = torch.from_numpy(ref.map.view(np.int32).copy()).cuda()
    D = cuda(ref.D.reshape(-1))
    want = ref.apply(src)
    want[ref.constrained] = 0.0  # the seam does not write identity rows
    dst = torch.zeros(ref.n_dofs, dtype=torch.float64, device="cuda")
    for gs in (2.0 ** -30, 1e-30, 1e30):  # aligned G: any scale
        dst.zero_()
        mf.bk5_lvector(3, D, cuda(ref.G * gs), cuda(src), dst, dmap, arith="df")
        assert rel(dst.cpu().numpy(), want * gs) <= TOL

    def unaligned(g):  # the same values 8 bytes past a 16-byte boundary
        buf = torch.zeros(g.size + 1, dtype=torch.float64, device="cuda")
        buf[1:] = cuda(g)
        return buf[1:]

    dst.zero_()
    mf.bk5_lvector(3, D, unaligned(ref.G * 2.0 ** -30), cuda(src), dst, dmap, arith="df")
    assert rel(dst.cpu().numpy(), want * 2.0 ** -30) <= TOL
    for g in (ref.G * 1e-30, ref.G * 1e30):
        dst.zero_()
        with pytest.raises(MfgbError) as e:
            mf.bk5_lvector(3, D, unaligned(g), cuda(src), dst, dmap, arith="df")
        assert e.value.status == _abi.ERR_RANGE


@pytest.mark.parametrize("p", [2, 4, 7])
def test_bk6_df_components_carry_own_scale(mf, orc, p):
    """BK6 scales every component of a cell on its own: components 1e-280,
    1 and 2^300 apart each meet the bar against the scaled oracle."""
    cells = (3, 4, 2)
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.1))
    ref = orc.BoxProblem(*cells, p, amplitude=0.1)
    base = np.random.default_rng(p + 40).uniform(-1, 1, 3 * ref.n_dofs)
    scales = (1e-280, 1.0, 2.0 ** 300)
    src = base.copy()
    for c, sc in enumerate(scales):
        src[c::3] *= sc
    import torch
    y = torch.zeros(3 * ref.n_dofs, dtype=torch.float64, device="cuda")
    A.vmult_vector(y, cuda(src), arith="df")
    mf.check_device_errors()
    got = y.cpu().numpy()
    for c, sc in enumerate(scales):
        assert rel(got[c::3], ref.apply(base[c::3]) * sc) <= TOL


@pytest.mark.parametrize("arith", ["df", "fp64"])
def test_nan_in_rhs_is_nonfinite(mf, arith):
    from benchmarks_gb300 import MfgbError, _abi
    A = mf.LaplaceOperator(mf.BoxMesh(4, 4, 4, degree=3, amplitude=0.05))
    b = A.rhs_uniform(3)
    b[A.m() // 2] = float("nan")
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(100, 1e-300, 1e-8)
    with pytest.raises(MfgbError) as e:
        mf.SolverCG(ctl).solve(A, x, b, A.get_matrix_diagonal_inverse(), arith=arith)
    assert e.value.status == _abi.ERR_NONFINITE
