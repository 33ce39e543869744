"""BK5 operator on the GPU (through the C ABI) against the CPU oracle.

Tolerance: relative 2-norm error <= 1e-12 for both kernel arithmetics (native
FP64 and double-float), the bar the operator must meet in FP64.
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
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def to_dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


CASES = [(1, (5, 4, 3), 0.05), (2, (3, 4, 2), 0.05), (3, (4, 3, 3), 0.1), (4, (3, 2, 3), 0.05),
         (5, (2, 3, 2), 0.15), (6, (2, 2, 2), 0.05), (7, (2, 1, 2), 0.1), (8, (1, 2, 2), 0.05)]


@pytest.mark.parametrize("p,cells,amp", CASES)
@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_vmult_matches_oracle(mf, orc, p, cells, amp, arith):
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=amp))
    ref = orc.BoxProblem(*cells, p, amplitude=amp)
    assert A.m() == ref.n_dofs and A.n_constrained == ref.constrained.size
    src = np.random.default_rng(p).uniform(-1, 1, ref.n_dofs)  # constrained entries nonzero too
    want = ref.apply(src)
    y = A.initialize_dof_vector()
    A.vmult(y, to_dev(src), arith=arith)
    got = y.cpu().numpy()
    assert rel(got, want) <= TOL
    np.testing.assert_array_equal(got[ref.constrained], src[ref.constrained])


@pytest.mark.parametrize("p", [1, 3, 4, 8])
def test_setup_matches_oracle(mf, orc, p):
    A = mf.LaplaceOperator(mf.BoxMesh(3, 2, 2, degree=p, amplitude=0.1))
    ref = orc.BoxProblem(3, 2, 2, p, amplitude=0.1)
    dof_map, G, cons = A.export()
    np.testing.assert_array_equal(dof_map, ref.map)
    np.testing.assert_array_equal(cons, ref.constrained)
    assert rel(G, ref.G) <= 1e-14


@pytest.mark.parametrize("p", range(1, 9))
@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_evector_seam_reference_cases(mf, orc, golden, p, arith):
    """E-vector seam against the reference's own serial kernel outputs."""
    import torch
    case = golden["random_cases"][str(p)]
    nq = p + 1
    nt = nq ** 3
    g = np.array(case["g"])
    nelmt = g.size // nt
    G = np.repeat(g.reshape(nelmt, 1, nt), 6, axis=1).reshape(-1)
    out = torch.zeros(nelmt * nt, dtype=torch.float64, device="cuda")
    mf.bk5_evector(p, to_dev(np.array(case["dbasis"])), to_dev(G), to_dev(np.array(case["in"])),
                   out, arith=arith)
    assert rel(out.cpu().numpy(), np.array(case["out"])) <= TOL
    # reference verification run: G = 2, in = 3, dbasis = cos, nelmt = 1000
    nelmt = 1000
    out = torch.zeros(nelmt * nt, dtype=torch.float64, device="cuda")
    mf.bk5_evector(p, to_dev(np.cos(np.arange(nq * nq, dtype=np.float64))),
                   torch.full((nelmt * 6 * nt,), 2.0, dtype=torch.float64, device="cuda"),
                   torch.full((nelmt * nt,), 3.0, dtype=torch.float64, device="cuda"), out,
                   arith=arith)
    norm = float(torch.linalg.norm(out))
    assert abs(norm - golden["verification_norms"][str(p)]) <= TOL * norm


@pytest.mark.parametrize("p", [2, 5])
@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_evector_seam_general_metric(mf, orc, p, arith):
    import torch
    nq = p + 1
    nt = nq ** 3
    rng = np.random.default_rng(5)
    nelmt = 37
    D = rng.uniform(-1, 1, nq * nq)
    G = rng.uniform(-1, 1, nelmt * 6 * nt)
    u = rng.uniform(-1, 1, nelmt * nt)
    out = torch.zeros(nelmt * nt, dtype=torch.float64, device="cuda")
    mf.bk5_evector(p, to_dev(D), to_dev(G), to_dev(u), out, arith=arith)
    assert rel(out.cpu().numpy(), orc.evector(nq, D, G, u)) <= TOL


@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_lvector_seam_and_array_setup(mf, orc, arith):
    """Kernel seam with caller-provided map/G, and the operator built from
    host arrays (the deal.II set-up path)."""
    import torch
    ref = orc.BoxProblem(3, 3, 2, 4, amplitude=0.1)
    src = np.random.default_rng(9).uniform(-1, 1, ref.n_dofs)
    dst = torch.zeros(ref.n_dofs, dtype=torch.float64, device="cuda")
    mf.bk5_lvector(4, to_dev(ref.D.reshape(-1)), to_dev(ref.G), to_dev(src), dst,
                   to_dev(ref.map.view(np.int32)), arith=arith)
    want = ref.apply(src)
    want[ref.constrained] = 0.0  # the seam does not write identity rows
    assert rel(dst.cpu().numpy(), want) <= TOL
    A = mf.LaplaceOperator(degree=4, n_dofs=ref.n_dofs, dof_map=ref.map, G=ref.G,
                           constrained=ref.constrained, arith=arith)
    y = A.initialize_dof_vector()
    A.vmult(y, to_dev(src))
    assert rel(y.cpu().numpy(), ref.apply(src)) <= TOL


@pytest.mark.parametrize("p", [1, 3, 6])
def test_diagonal_matches_oracle(mf, orc, p):
    A = mf.LaplaceOperator(mf.BoxMesh(3, 2, 3, degree=p, amplitude=0.1))
    ref = orc.BoxProblem(3, 2, 3, p, amplitude=0.1)
    d = A.compute_diagonal().cpu().numpy()
    assert rel(d, ref.diagonal()) <= 1e-13
    inv = A.get_matrix_diagonal_inverse().get_vector().cpu().numpy()
    assert rel(inv, orc.invert_diagonal(ref.diagonal())) <= 1e-13
    assert A.el(5, 5) == pytest.approx(d[5])


def test_rhs_bit_exact(mf, orc):
    A = mf.LaplaceOperator(mf.BoxMesh(5, 4, 3, degree=2))
    ref = orc.BoxProblem(5, 4, 3, 2)
    for seed in (0, 1, 12345):
        np.testing.assert_array_equal(A.rhs_uniform(seed).cpu().numpy(), ref.rhs(seed))


def test_edge_cases(mf, orc):
    import torch
    from benchmarks_gb300 import MfgbError
    # single p=1 cell: every DoF is constrained -> identity
    A = mf.LaplaceOperator(mf.BoxMesh(1, 1, 1, degree=1))
    assert A.m() == 8 and A.n_constrained == 8
    x = torch.arange(8, dtype=torch.float64, device="cuda")
    y = A.initialize_dof_vector()
    A.vmult(y, x)
    assert torch.equal(x, y)
    # dst aliasing src is rejected
    with pytest.raises(MfgbError):
        A.vmult(x, x)
    # operator with no cells: identity on the constrained list, zero elsewhere
    B = mf.LaplaceOperator(degree=2, n_dofs=5, dof_map=np.zeros(0, np.uint32), G=np.zeros(0),
                           constrained=np.array([1, 3]))
    z = torch.ones(5, dtype=torch.float64, device="cuda")
    w = torch.full((5,), 7.0, dtype=torch.float64, device="cuda")
    B.vmult(w, z)
    assert w.cpu().tolist() == [0.0, 1.0, 0.0, 1.0, 0.0]
    # out-of-range map entries and degrees are rejected on the host
    with pytest.raises(MfgbError):
        mf.LaplaceOperator(degree=1, n_dofs=4, dof_map=np.full(8, 9, np.uint32), G=np.zeros(48))
    with pytest.raises(MfgbError):
        mf.LaplaceOperator(mf.BoxMesh(1, 1, 1, degree=0))


def test_full_size_properties(mf):
    """BK5 at the bench size (p = 4, 128 x 128 x 64 cells, 67,634,433 DoFs):
    size-independent properties -- the two arithmetics agree to 1e-12,
    linearity, symmetry, positivity."""
    import torch
    A = mf.LaplaceOperator(mf.BoxMesh(128, 128, 64, degree=4, amplitude=0.05))
    assert A.m() == 67634433
    u = A.rhs_uniform(1)
    v = A.rhs_uniform(2)
    Au64, Audf = A.initialize_dof_vector(), A.initialize_dof_vector()
    A.vmult(Au64, u, arith="fp64")
    A.vmult(Audf, u, arith="df")
    assert float(torch.linalg.norm(Au64 - Audf) / torch.linalg.norm(Au64)) <= TOL
    Av, Auv = A.initialize_dof_vector(), A.initialize_dof_vector()
    A.vmult(Av, v)
    A.vmult(Auv, u + 2.0 * v)
    # linear to the arithmetic's precision (about 2^-43 normwise)
    assert float(torch.linalg.norm(Auv - (Audf + 2.0 * Av)) / torch.linalg.norm(Auv)) <= TOL
    uAv, vAu = mf.dot(u, Av), mf.dot(v, Audf)
    assert abs(uAv - vAu) <= 1e-12 * abs(uAv)
    assert mf.dot(u, Audf) > 0
    del A
    torch.cuda.empty_cache()


@pytest.mark.parametrize("shape", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("p", [1, 2, 4, 5, 7, 8])
def test_every_kernel_shape_matches_oracle(mf, orc, shape, arith, p):
    """Each thread layout (column, point, column + TMA prefetch) for each
    arithmetic, on a mesh whose cell count leaves a partial last batch."""
    import ctypes
    from benchmarks_gb300 import _abi
    L = mf.lib()
    a = mf._arith(arith)
    old = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(a, p, ctypes.byref(old)))
    try:
        _abi.check(L.mfgb_set_kernel_shape(a, p, shape))
        cells = (3, 5, 3)  # 45 cells: not a multiple of any batch size
        A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.1))
        ref = orc.BoxProblem(*cells, p, amplitude=0.1)
        src = np.random.default_rng(3).uniform(-1, 1, ref.n_dofs)
        y = A.initialize_dof_vector()
        A.vmult(y, to_dev(src), arith=arith)
        assert rel(y.cpu().numpy(), ref.apply(src)) <= TOL
        # the energy (p.Ap) variant used by CG: iterate after 6 steps (before
        # convergence, so the comparison is not at a rounding-level residual)
        b = A.rhs_uniform(4)
        x = A.initialize_dof_vector()
        ctl = mf.ReductionControl(6, 1e-300, 1e-14)
        with pytest.raises(mf.MfgbError):
            mf.SolverCG(ctl).solve(A, x, b, arith=arith)
        x_ref, info = ref.cg(ref.rhs(4), reduce=1e-14, max_steps=6)
        assert ctl.last_step() == info["steps"] == 6
        assert rel(x.cpu().numpy(), x_ref) <= 1e-10
        _abi.check(L.mfgb_check_device_errors(None))
    finally:
        _abi.check(L.mfgb_set_kernel_shape(a, p, old.value))


@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
@pytest.mark.parametrize("arith", ["fp64", "df"])
def test_bk6_vector_operator(mf, orc, p, arith):
    """BK6: every interleaved component goes through the scalar operator."""
    cells = (3, 4, 2)
    A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.1))
    ref = orc.BoxProblem(*cells, p, amplitude=0.1)
    src = np.random.default_rng(p + 10).uniform(-1, 1, 3 * ref.n_dofs)
    y = torch_zeros(3 * ref.n_dofs)
    A.vmult_vector(y, to_dev(src), arith=arith)
    got = y.cpu().numpy()
    want = np.empty_like(src)
    for c in range(3):
        want[c::3] = ref.apply(src[c::3])
    assert rel(got, want) <= TOL


def torch_zeros(n):
    import torch
    return torch.zeros(n, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("shape", [0, 2, 3, 4])
@pytest.mark.parametrize("p", [2, 4, 5, 8])
def test_fp32_tma_tail_batch(mf, orc, p, shape):
    """FP32 geometric factors in an odd last batch (a 4-byte tile that is not a
    16-byte multiple) go through plain loads: correct result, no timeout."""
    import ctypes
    import torch
    from benchmarks_gb300 import _abi
    L = mf.lib()
    old = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(2, p, ctypes.byref(old)))
    try:
        _abi.check(L.mfgb_set_kernel_shape(2, p, shape))
        cells = (3, 3, 3)  # 27 cells: odd last batch for every batch size
        A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=p, amplitude=0.1))
        ref = orc.BoxProblem(*cells, p, amplitude=0.1)
        src = np.random.default_rng(1).uniform(-1, 1, ref.n_dofs)
        s32 = torch.from_numpy(src.astype(np.float32)).cuda()
        d32 = torch.zeros_like(s32)
        _abi.check(L.mfgb_vmult_f32(A.handle, ctypes.c_void_p(d32.data_ptr()),
                                    ctypes.c_void_p(s32.data_ptr()), mf._stream_ptr()))
        _abi.check(L.mfgb_check_device_errors(None))
        assert rel(d32.cpu().numpy().astype(np.float64), ref.apply(src)) <= 1e-5
    finally:
        _abi.check(L.mfgb_set_kernel_shape(2, p, old.value))


def test_autotune_small(mf, tmp_path):
    """The autotuner times each shape, restores the table, and round-trips."""
    import ctypes
    from benchmarks_gb300 import _abi, autotune
    L = mf.lib()
    before = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(1, 3, ctypes.byref(before)))
    r = autotune.tune(degrees=[3], ariths=("df", "fp32"), target_dofs=2e5, reps=2, apply=False)
    after = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(1, 3, ctypes.byref(after)))
    assert after.value == before.value
    for name in ("df", "fp32"):
        e = r[name][3]
        shapes = autotune.shapes_for(autotune.ARITHS[name])
        assert e["best"] in shapes and len(e["ms"]) == len(shapes) and min(e["ms"]) > 0
    path = tmp_path / "tune.json"
    autotune.save(r, path)
    r2 = autotune.load(path, apply=False)
    assert r2["df"]["3"]["best"] == r["df"][3]["best"]


@pytest.mark.parametrize("arith", ["df", "fp64"])
@pytest.mark.parametrize("form", ["gll", "gauss", "helmholtz", "bp3"])
def test_vmult_host_pipeline(mf, orc, form, arith):
    """The host-buffer apply (slab-pipelined copies) equals the device vmult, with
    the identity rows copied exactly, for several slab layouts and repeated calls."""
    import torch
    for cells in ((3, 2, 9), (2, 3, 1), (4, 4, 16)):
        A = mf.LaplaceOperator(mf.BoxMesh(*cells, degree=3, amplitude=0.06), arith=arith,
                               quadrature=form)
        src = torch.from_numpy(np.random.default_rng(sum(cells)).uniform(-1, 1, A.m()))
        h_src = src.pin_memory()
        h_dst = torch.empty_like(h_src).pin_memory()
        want = A.initialize_dof_vector()
        A.vmult(want, src.cuda())
        for _ in range(2):
            h_dst.fill_(float("nan"))
            A.vmult_host(h_dst, h_src)
            torch.cuda.synchronize()
            assert rel(h_dst.numpy(), want.cpu().numpy()) <= 1e-14
        cons = orc.BoxProblem(*cells, 3).constrained
        assert np.array_equal(h_dst.numpy()[cons], src.numpy()[cons])


def test_vmult_host_array_operator(mf, orc):
    import torch
    ref = orc.BoxProblem(3, 2, 2, 2, amplitude=0.05)
    A = mf.LaplaceOperator(degree=2, n_dofs=ref.n_dofs, dof_map=ref.map, G=ref.G,
                           constrained=ref.constrained)
    src = np.random.default_rng(0).uniform(-1, 1, ref.n_dofs)
    h_dst = torch.empty(ref.n_dofs, dtype=torch.float64).pin_memory()
    A.vmult_host(h_dst, torch.from_numpy(src).pin_memory())
    torch.cuda.synchronize()
    assert rel(h_dst.numpy(), ref.apply(src)) <= 1e-12


def test_vmult_dummy(mf):
    """vmult_dummy(ghost_on, compute_on) composes to vmult; compute alone leaves
    the constrained rows at the cell-loop value, ghost alone only sets them."""
    import torch
    A = mf.LaplaceOperator(mf.BoxMesh(3, 3, 3, degree=2, amplitude=0.05))
    src = A.rhs_uniform(2) + 1.0
    want = A.initialize_dof_vector()
    A.vmult(want, src)
    y = A.initialize_dof_vector()
    A.vmult_dummy(y, src, True, True)
    assert torch.equal(y, want) or float(torch.linalg.norm(y - want)) <= 1e-14 * float(torch.linalg.norm(want))
    z = A.initialize_dof_vector()
    A.vmult_dummy(z, src, False, True)
    A.vmult_dummy(z, src, True, False)
    assert float(torch.linalg.norm(z - want)) <= 1e-14 * float(torch.linalg.norm(want))
