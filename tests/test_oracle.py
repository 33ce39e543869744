"""CPU oracle pinned against the reference's own CPU code and known answers."""
import numpy as np
import pytest


@pytest.mark.parametrize("p", range(1, 9))
def test_reference_verification_norm(orc, golden, p):
    """CEED_BK/src/BK5/serial_verification.cc: G = 2, in = 3, dbasis = cos."""
    nq = p + 1
    nt = nq ** 3
    nelmt = 1000
    D = np.cos(np.arange(nq * nq, dtype=np.float64))
    G = np.full(nelmt * 6 * nt, 2.0)
    u = np.full(nelmt * nt, 3.0)
    y = orc.evector(nq, D, G, u)
    want = golden["verification_norms"][str(p)]
    assert np.sqrt(np.sum(y * y)) == pytest.approx(want, rel=1e-13)


@pytest.mark.parametrize("p", range(1, 9))
def test_reference_serial_random(orc, golden, p):
    case = golden["random_cases"][str(p)]
    nq = p + 1
    nt = nq ** 3
    g = np.array(case["g"])
    nelmt = g.size // nt
    G = np.repeat(g.reshape(nelmt, 1, nt), 6, axis=1).reshape(-1)
    y = orc.evector(nq, np.array(case["dbasis"]), G, np.array(case["in"]))
    want = np.array(case["out"])
    assert np.max(np.abs(y - want)) <= 1e-13 * np.max(np.abs(want))


@pytest.mark.parametrize("p", range(1, 9))
def test_lagrange_derivative_matches_reference(orc, golden, p):
    case = golden["lagrange_D"][str(p)]
    x, _ = orc.gll(p + 1)
    np.testing.assert_allclose(x, case["nodes"], rtol=0, atol=1e-15)
    D = orc.derivative_matrix(x)
    np.testing.assert_allclose(D, np.array(case["D"]), rtol=1e-14, atol=1e-13)


def test_lagrange_partition_of_unity(orc):
    """sum_factorization/tests/test_lagrange.cc:18-47 (nodes and sweep as there)."""
    for nodes in ([-2.0, 0.5], [-2.0, 0.0, 1.0], [-3.0, 0.5, 1.0, 1.5]):
        nd = np.array(nodes)
        total = 0.0
        for x in np.arange(-2.0, 0.5 + 1e-9, 0.05):
            total += sum(orc.lib().orc_lagrange_value(len(nodes), orc._p(nd), j, float(x))
                         for j in range(len(nodes))) - 1.0
        assert abs(total) < 1e-6


@pytest.mark.parametrize("p", range(1, 9))
def test_gll_quadrature_exactness(orc, p):
    x, w = orc.gll(p + 1)
    assert np.all(np.diff(x) > 0) and x[0] == -1.0 and x[-1] == 1.0
    for k in range(0, 2 * p):  # GLL with p+1 points is exact up to degree 2p-1
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.dot(w, x ** k) - exact) < 1e-14
    # derivative matrix differentiates polynomials of degree <= p exactly
    D = orc.derivative_matrix(x)
    for k in range(0, p + 1):
        np.testing.assert_allclose(D @ x ** k, k * x ** max(k - 1, 0) if k else 0 * x,
                                   atol=1e-12)


def test_gauss_points(orc):
    for n in range(1, 10):
        x, w = orc.gauss(n)
        for k in range(0, 2 * n):
            exact = 0.0 if k % 2 else 2.0 / (k + 1)
            assert abs(np.dot(w, x ** k) - exact) < 1e-14


def test_mt19937_64_known_answer(orc):
    # the C++ standard's check value: 10000th output of mt19937_64 seeded 5489
    assert orc.mt19937_64_nth(5489, 10000) == 9981545732273789042


def test_rhs_uniform_range_and_constraints(orc):
    prob = orc.BoxProblem(3, 2, 2, 2)
    b = prob.rhs(11)
    assert np.all(b[prob.constrained] == 0.0)
    free = np.setdiff1d(np.arange(prob.n_dofs), prob.constrained)
    assert np.all((b[free] >= -1.0) & (b[free] < 1.0))
    assert np.array_equal(b, prob.rhs(11)) and not np.array_equal(b, prob.rhs(12))


def test_box_mesh_counts_and_map(orc):
    prob = orc.BoxProblem(3, 4, 5, 2)
    assert prob.n_dofs == 7 * 9 * 11 and prob.n_cells == 60
    assert prob.constrained.size == 7 * 9 * 11 - 5 * 7 * 9
    valid = prob.map[prob.map != orc.INVALID_DOF]
    assert valid.max() < prob.n_dofs
    assert np.intersect1d(valid, prob.constrained).size == 0
    assert prob.n_bad_cells == 0


def test_shared_nodes_coincide(orc):
    """Deformed Q_p geometry stays conforming: shared GLL nodes of neighbours match."""
    prob = orc.BoxProblem(2, 1, 1, 3, amplitude=0.1)
    a, b = prob.cell_nodes(0).reshape(4, 4, 4, 3), prob.cell_nodes(1).reshape(4, 4, 4, 3)
    np.testing.assert_array_equal(a[:, :, -1, :], b[:, :, 0, :])


@pytest.mark.parametrize("p", [1, 2, 3, 5])
def test_geometry_matches_dense_stiffness(orc, p):
    """G = JxW Jinv Jinv^T with the reference-index order: the E-vector operator
    of an affinely sheared cell equals a dense stiffness matrix built directly
    from physical gradients J^{-T} grad_xi phi at the GLL points."""
    n = p + 1
    x, w = orc.gll(n)
    D = orc.derivative_matrix(x)
    M = np.array([[0.7, 0.2, -0.1], [0.15, 0.9, 0.25], [-0.05, 0.3, 1.1]])
    c0 = np.array([0.3, -0.2, 0.5])
    xyz = np.zeros((n ** 3, 3))
    for i in range(n):
        for j in range(n):
            for k in range(n):
                xyz[i * n * n + j * n + k] = M @ np.array([x[i], x[j], x[k]]) + c0
    G = np.zeros(6 * n ** 3)
    orc.lib().orc_cell_geometry(n, orc._p(D), orc._p(w), orc._p(np.ascontiguousarray(xyz)),
                                orc._p(G))
    K = np.zeros((n ** 3, n ** 3))
    for col in range(n ** 3):
        e = np.zeros(n ** 3); e[col] = 1.0
        K[:, col] = orc.evector(n, D, G, e)
    Jinv_T = np.linalg.inv(M).T
    det = abs(np.linalg.det(M))
    Kd = np.zeros_like(K)
    for a in range(n):
        for b in range(n):
            for c in range(n):
                grads = np.zeros((n ** 3, 3))
                for i in range(n):
                    for j in range(n):
                        for k in range(n):
                            l = i * n * n + j * n + k
                            grads[l] = [D[a, i] * (j == b) * (k == c), (i == a) * D[b, j] * (k == c),
                                        (i == a) * (j == b) * D[c, k]]
                phys = grads @ Jinv_T.T
                Kd += w[a] * w[b] * w[c] * det * phys @ phys.T
    np.testing.assert_allclose(K, Kd, rtol=1e-12, atol=1e-12 * np.abs(Kd).max())


def test_operator_symmetric_positive(orc):
    prob = orc.BoxProblem(3, 3, 2, 3, amplitude=0.08)
    u, v = prob.rhs(1), prob.rhs(2)
    Au, Av = prob.apply(u), prob.apply(v)
    assert abs(u @ Av - v @ Au) <= 1e-12 * abs(u @ Av)
    assert u @ Au > 0
    # identity rows on constrained DoFs
    z = np.random.default_rng(0).uniform(-1, 1, prob.n_dofs)
    np.testing.assert_array_equal(prob.apply(z)[prob.constrained], z[prob.constrained])


def test_diagonal_matches_operator_columns(orc):
    prob = orc.BoxProblem(2, 2, 2, 2, amplitude=0.1)
    d = prob.diagonal()
    for i in range(prob.n_dofs):
        e = np.zeros(prob.n_dofs); e[i] = 1.0
        assert abs(prob.apply(e)[i] - d[i]) <= 1e-13 * max(1.0, abs(d[i]))
    inv = orc.invert_diagonal(np.array([2.0, 0.0, -1.0]))
    np.testing.assert_array_equal(inv, [0.5, 1.0, 1.0])


def test_cg_converges_and_counts(orc):
    prob = orc.BoxProblem(4, 4, 4, 3)
    b = prob.rhs(3)
    x, info = prob.cg(b, reduce=1e-8)
    assert info["converged"] and info["last"] <= 1e-8 * info["initial"]
    r = b - prob.apply(x)
    assert np.linalg.norm(r) <= 1.01e-8 * info["initial"]
    xj, infoj = prob.cg(b, diag_inv=orc.invert_diagonal(prob.diagonal()), reduce=1e-8)
    assert infoj["converged"] and infoj["steps"] <= info["steps"]
    x2, info2 = prob.cg(b, reduce=1e-8, max_steps=3)
    assert not info2["converged"] and info2["steps"] == 3


def test_published_bp5_cg_counts(orc):
    """The reference's published BP5-variant CG runs (FE_Q(4), QGauss(5),
    f = 1, identity preconditioner, ReductionControl(1e9, 1e-16, 1e-9)):
    identical iteration counts and cg_reduction on cycles 8..12
    (bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/results/1_GPU.out:640-644)."""
    import json
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "published_bp5_cg.json")
    rows = {r["dofs"]: r for r in json.load(open(path))["rows"]}
    for cycle in range(8, 13):
        cells, lo, hi = orc.reference_scaling_mesh(cycle, 4)
        P = orc.GaussProblem(*cells, 4, lo=lo, hi=hi)
        pub = rows[P.n_dofs]
        assert P.n_cells == pub["cells"]
        _, info = P.cg(P.rhs_unit())
        assert info["steps"] == pub["cg_its"]
        red = (info["last"] / info["initial"]) ** (1.0 / info["steps"])
        assert f"{red:.3e}" == f"{pub['cg_reduction']:.3e}"


def test_gauss_operator_is_exact_stiffness_on_affine_cells(orc):
    """With nq = p + 1 Gauss points the operator on an affine cube equals the
    exactly integrated stiffness matrix: its energy of a polynomial of degree
    <= p is the exact Dirichlet integral."""
    P = orc.GaussProblem(2, 2, 2, 3, lo=(0, 0, 0), hi=(1, 1, 1))
    # u = x y z (1-x)(1-y)(1-z)-like interior polynomial sampled at the nodes is
    # not degree 3 per direction; use u = x(1-x) y(1-y) z(1-z), degree 2 each
    xyz = np.zeros((P.n_dofs, 3))
    for e in range(P.n_cells):
        nodes = P.cell_nodes(e)
        m = P.map[e * 64:(e + 1) * 64]
        valid = m != orc.INVALID_DOF
        xyz[m[valid].astype(np.int64)] = nodes[valid]
    x, y, z = xyz.T
    u = x * (1 - x) * y * (1 - y) * z * (1 - z)
    u[P.constrained] = 0.0
    energy = u @ P.apply(u)
    # exact: integral |grad u|^2 = 3 * (1/3) * (1/30)^2
    assert abs(energy - 3 * (1 / 3) * (1 / 30) ** 2) <= 1e-13


@pytest.mark.parametrize("p", range(1, 9))
def test_bk1_bk3_match_reference_serial(orc, golden13, p):
    """The oracle's BK1 / BK3 E-vector operators against the reference's serial
    kernels (random basis, dbasis, JxW, six independent G components)."""
    nq, nm = p + 2, p + 1
    c = golden13["bk1_cases"][str(p)]
    y = orc.bk1_evector(nm, nq, np.array(c["basis"]), np.array(c["JxW"]), np.array(c["in"]))
    assert np.linalg.norm(y - c["out"]) <= 1e-13 * np.linalg.norm(c["out"])
    c = golden13["bk3_cases"][str(p)]
    y = orc.bk3_evector(nm, nq, np.array(c["basis"]), np.array(c["dbasis"]), np.array(c["G"]),
                        np.array(c["in"]))
    assert np.linalg.norm(y - c["out"]) <= 1e-13 * np.linalg.norm(c["out"])


@pytest.mark.parametrize("p", [1, 4, 8])
def test_bk1_bk3_verification_norms(orc, golden13, p):
    """CEED_BK/src/BK{1,3}/serial_verification.cc inputs (cos bases, in = 3,
    JxW = 1, G = 2, 1000 elements): the printed norms."""
    nq, nm, nel = p + 2, p + 1, 1000
    basis = np.cos(np.arange(nq * nm, dtype=float))
    dbasis = np.cos(np.arange(nq * nq, dtype=float))
    u = np.full(nel * nm ** 3, 3.0)
    n1 = np.linalg.norm(orc.bk1_evector(nm, nq, basis, np.ones(nel * nq ** 3), u))
    n3 = np.linalg.norm(orc.bk3_evector(nm, nq, basis, dbasis, np.full(nel * 6 * nq ** 3, 2.0), u))
    assert n1 == pytest.approx(golden13["bk1_norms"][str(p)], rel=1e-12)
    assert n3 == pytest.approx(golden13["bk3_norms"][str(p)], rel=1e-12)


def test_helmholtz_mass_term_and_diagonal(orc):
    """Helmholtz = stiffness + mass at QGauss(p+1): on an affine cube the mass
    part integrates v^2 exactly for the bubble v = x(1-x) y(1-y) z(1-z); the
    diagonal equals the operator's own diagonal entries."""
    H = orc.HelmholtzProblem(2, 2, 3, 2, amplitude=0.0)
    K = orc.GaussProblem(2, 2, 3, 2, amplitude=0.0)
    free = np.setdiff1d(np.arange(H.n_dofs), H.constrained)
    # nodal coordinates of the lexicographic GLL nodes (x fastest)
    xg, _ = orc.gll(3)
    def axis(n):
        return np.concatenate([[0.0]] + [c / n + (xg[1:] + 1) / (2 * n) for c in range(n)])
    X, Y, Z = np.meshgrid(axis(2), axis(2), axis(3), indexing="ij")
    v = (X * (1 - X) * Y * (1 - Y) * Z * (1 - Z)).transpose(2, 1, 0).reshape(-1)
    mass = v @ (H.apply(v) - K.apply(v))
    assert mass == pytest.approx((1 / 30) ** 3, rel=1e-12)
    d = H.diagonal()
    for i in free[:: max(1, free.size // 15)]:
        e = np.zeros(H.n_dofs)
        e[i] = 1.0
        assert d[i] == pytest.approx(H.apply(e)[i], rel=1e-12)
    assert np.all(d[H.constrained] == 1.0)
    # symmetric positive definite on the free DoFs
    u, w = np.random.default_rng(0).uniform(-1, 1, (2, H.n_dofs))
    u[H.constrained] = w[H.constrained] = 0
    assert u @ H.apply(w) == pytest.approx(w @ H.apply(u), rel=1e-12)
    assert u @ H.apply(u) > 0


@pytest.mark.parametrize("nq_extra, mass", [(0, False), (1, False), (0, True)])
def test_gauss_diagonal_sum_factorisation(orc, nq_extra, mass):
    """The factorised form of the Gauss-point diagonal that the GPU kernel
    evaluates (seven quadrature sums, each contracted one direction at a time
    with B^2, (DB)^2 or B DB; factor 2 on the three cross terms) equals the
    oracle's direct sum over the quadrature points."""
    p = 3
    cls = orc.HelmholtzProblem if mass else orc.GaussProblem
    if mass:  # Helmholtz: q = p + 1
        P = cls(2, 3, 2, p, amplitude=0.08)
    else:
        P = cls(2, 3, 2, p, nq=p + 1 + nq_extra, amplitude=0.08)
    n, q = P.n, P.nq
    B, DG = P.B, P.DG
    DB = DG @ B
    w = {0: B * B, 1: DB * DB, 2: B * DB}  # [q][n]
    kinds = [(1, 0, 0, 1.0), (2, 2, 0, 2.0), (2, 0, 2, 2.0), (0, 1, 0, 1.0), (0, 2, 2, 2.0),
             (0, 0, 1, 1.0)]  # rr rs rt ss st tt: (i, j, k) weight kinds, factor
    G = P.Gg.reshape(P.n_cells, 6, q, q, q)
    diag = np.zeros(P.n_dofs)
    for e in range(P.n_cells):
        de = np.zeros((n, n, n))
        for T, (ki, kj, kk, f) in enumerate(kinds):
            de += f * np.einsum("ia,jb,kc,ijk->abc", w[ki], w[kj], w[kk], G[e, T])
        if mass:
            W = P.JxW.reshape(P.n_cells, q, q, q)[e]
            de += np.einsum("ia,jb,kc,ijk->abc", w[0], w[0], w[0], W)
        idx = P.map.reshape(P.n_cells, n ** 3)[e].astype(np.int64)
        ok = idx != 0xFFFFFFFF  # Dirichlet DoFs are masked out of the map
        np.add.at(diag, idx[ok], de.reshape(-1)[ok])
    diag[P.constrained] = 1.0
    direct = np.zeros(P.n_dofs)
    orc._gauss_sigs().orc_gauss_diagonal(n, q, orc._p(B), orc._p(DG), P.n_cells, orc._p(P.map),
                                         orc._p(P.Gg), orc._p(P.JxW) if mass else None, P.n_dofs,
                                         P.constrained.size, orc._p(P.constrained), orc._p(direct))
    assert np.max(np.abs(diag - direct)) <= 1e-13 * np.max(np.abs(direct))
