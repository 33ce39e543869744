"""CEED BK1 (mass) and BK3 (Laplacian, q = p + 2) E-vector seams on the GPU
against the reference's serial outputs and the CPU oracle.  Tolerance: 1e-12
relative for the three FP64 arithmetics (DFMA, double-float on the FP32
pipes, DMMA tensor-core tiles for BK1)."""
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


def cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def rel(a, b):
    """|a - b| / |b|, both divided by max|b| first: the squares inside the norms
    of vectors near 1e-280 would underflow to zero"""
    m = float(np.max(np.abs(b)))
    if m == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.linalg.norm((a - b) / m) / np.linalg.norm(b / m))


@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("p", range(1, 9))
def test_bk1_bk3_reference_cases(mf, golden13, p, arith):
    import torch
    c = golden13["bk1_cases"][str(p)]
    u = cuda(c["in"])
    y = torch.zeros_like(u)
    mf.bk1_evector(p, cuda(c["basis"]), cuda(c["JxW"]), u, y, arith=arith)
    assert rel(y.cpu().numpy(), np.array(c["out"])) <= 1e-12
    c = golden13["bk3_cases"][str(p)]
    u = cuda(c["in"])
    y = torch.zeros_like(u)
    mf.bk3_evector(p, cuda(c["basis"]), cuda(c["dbasis"]), cuda(c["G"]), u, y, arith=arith)
    assert rel(y.cpu().numpy(), np.array(c["out"])) <= 1e-12


@pytest.mark.parametrize("arith", ["fp64", "df"])
@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
def test_bk1_bk3_many_elements_match_oracle(mf, orc, p, arith):
    """Ragged element counts (a partial last batch) on Gauss-Lobatto-to-Gauss
    bases and SPD per-point metrics."""
    import torch
    nq, nm = p + 2, p + 1
    g = np.random.default_rng(p)
    nel = 37
    xg, _ = orc.gll(nm)
    xq, _ = orc.gauss(nq)
    basis = orc.interpolation_matrix(xg, xq)
    dbasis = orc.derivative_matrix(xq)
    jxw = g.uniform(0.5, 2.0, nel * nq ** 3)
    G = g.uniform(-0.3, 0.3, (nel, 6, nq ** 3))
    G[:, 0] += 2.0
    G[:, 3] += 2.0
    G[:, 5] += 2.0
    u = g.uniform(-1, 1, nel * nm ** 3)
    y1 = torch.zeros(u.size, dtype=torch.float64, device="cuda")
    mf.bk1_evector(p, cuda(basis), cuda(jxw), cuda(u), y1, arith=arith)
    assert rel(y1.cpu().numpy(), orc.bk1_evector(nm, nq, basis, jxw, u)) <= 1e-12
    y3 = torch.zeros_like(y1)
    mf.bk3_evector(p, cuda(basis), cuda(dbasis), cuda(G.reshape(-1)), cuda(u), y3, arith=arith)
    assert rel(y3.cpu().numpy(), orc.bk3_evector(nm, nq, basis, dbasis, G.reshape(-1), u)) <= 1e-12


@pytest.mark.parametrize("p", range(1, 7))
def test_bk1_tensor_cores_match_reference_and_oracle(mf, golden13, orc, p):
    """The FP64 tensor-core BK1 (mma m8n8k4 .f64 tiles) on the reference's own
    serial outputs and on 37 / 1000 elements against the oracle: the grid
    strides over warps, so a partial last CTA and several elements per warp
    are both exercised."""
    import torch
    c = golden13["bk1_cases"][str(p)]
    u = cuda(c["in"])
    y = torch.zeros_like(u)
    mf.bk1_evector(p, cuda(c["basis"]), cuda(c["JxW"]), u, y, arith="tc")
    assert rel(y.cpu().numpy(), np.array(c["out"])) <= 1e-12
    nq, nm = p + 2, p + 1
    g = np.random.default_rng(10 + p)
    xg, _ = orc.gll(nm)
    xq, _ = orc.gauss(nq)
    basis = orc.interpolation_matrix(xg, xq)
    for nel in (37, 1000):
        jxw = g.uniform(0.5, 2.0, nel * nq ** 3)
        u = g.uniform(-1, 1, nel * nm ** 3)
        y = torch.zeros(u.size, dtype=torch.float64, device="cuda")
        mf.bk1_evector(p, cuda(basis), cuda(jxw), cuda(u), y, arith="tc")
        assert rel(y.cpu().numpy(), orc.bk1_evector(nm, nq, basis, jxw, u)) <= 1e-12


def test_bk1_tensor_cores_large_grid(mf):
    """More elements than one wave of warps: agreement with the DFMA kernel
    element by element."""
    import torch
    p, nel = 4, 300000
    nq, nm = p + 2, p + 1
    g = torch.Generator(device="cuda").manual_seed(3)
    basis = torch.rand(nq * nm, dtype=torch.float64, device="cuda", generator=g)
    jxw = torch.rand(nel * nq ** 3, dtype=torch.float64, device="cuda", generator=g)
    u = torch.rand(nel * nm ** 3, dtype=torch.float64, device="cuda", generator=g) - 0.5
    y0, y1 = torch.zeros_like(u), torch.zeros_like(u)
    mf.bk1_evector(p, basis, jxw, u, y0, arith="fp64")
    mf.bk1_evector(p, basis, jxw, u, y1, arith="tc")
    d = (y1 - y0).view(nel, -1).norm(dim=1) / y0.view(nel, -1).norm(dim=1)
    assert float(d.max()) <= 1e-12


@pytest.mark.parametrize("p", [2, 5, 8])
def test_bk1_df_carries_any_scale(mf, orc, p):
    """The double-float BK1 seam scales every element's input and JxW by powers
    of two: inputs and weights far outside the float range, and exact zeros,
    meet the 1e-12 bar."""
    import torch
    nq, nm = p + 2, p + 1
    g = np.random.default_rng(40 + p)
    nel = 53
    xg, _ = orc.gll(nm)
    xq, _ = orc.gauss(nq)
    basis = orc.interpolation_matrix(xg, xq)
    jxw = g.uniform(0.5, 2.0, nel * nq ** 3)
    u = g.uniform(-1, 1, nel * nm ** 3)
    u[::9] = 0.0
    want = orc.bk1_evector(nm, nq, basis, jxw, u)
    for su, sj in ((1e-280, 1.0), (2.0 ** 300, 2.0 ** -100), (1e-30, 1e30)):
        y = torch.zeros(u.size, dtype=torch.float64, device="cuda")
        mf.bk1_evector(p, cuda(basis), cuda(jxw * sj), cuda(u * su), y, arith="df")
        assert rel(y.cpu().numpy(), want * su * sj) <= 1e-12


@pytest.mark.parametrize("p", [2, 5, 8])
def test_bk3_df_carries_any_scale(mf, orc, p):
    """The double-float BK3 seam scales every element's input and G by powers
    of two: both far outside the float range meet the 1e-12 bar."""
    import torch
    nq, nm = p + 2, p + 1
    g = np.random.default_rng(50 + p)
    nel = 41
    xg, _ = orc.gll(nm)
    xq, _ = orc.gauss(nq)
    basis = orc.interpolation_matrix(xg, xq)
    dbasis = orc.derivative_matrix(xq)
    G = g.uniform(-0.3, 0.3, (nel, 6, nq ** 3))
    G[:, 0] += 2.0
    G[:, 3] += 2.0
    G[:, 5] += 2.0
    u = g.uniform(-1, 1, nel * nm ** 3)
    u[::11] = 0.0
    want = orc.bk3_evector(nm, nq, basis, dbasis, G.reshape(-1), u)
    for su, sg in ((1e-280, 1.0), (2.0 ** 300, 2.0 ** -100), (1e-30, 1e30)):
        y = torch.zeros(u.size, dtype=torch.float64, device="cuda")
        mf.bk3_evector(p, cuda(basis), cuda(dbasis), cuda(G.reshape(-1) * sg), cuda(u * su), y,
                       arith="df")
        assert rel(y.cpu().numpy(), want * su * sg) <= 1e-12


def test_bk_verification_norms_on_gpu(mf, golden13):
    import torch
    p, nel = 4, 1000
    nq, nm = p + 2, p + 1
    basis = cuda(np.cos(np.arange(nq * nm, dtype=float)))
    dbasis = cuda(np.cos(np.arange(nq * nq, dtype=float)))
    u = cuda(np.full(nel * nm ** 3, 3.0))
    y = torch.zeros_like(u)
    mf.bk1_evector(p, basis, cuda(np.ones(nel * nq ** 3)), u, y)
    assert float(torch.linalg.norm(y)) == pytest.approx(golden13["bk1_norms"][str(p)], rel=1e-12)
    mf.bk3_evector(p, basis, dbasis, cuda(np.full(nel * 6 * nq ** 3, 2.0)), u, y, arith="df")
    assert float(torch.linalg.norm(y)) == pytest.approx(golden13["bk3_norms"][str(p)], rel=1e-12)


def test_bkq_invalid_arguments(mf):
    from benchmarks_gb300 import _abi
    L = mf.lib()
    assert L.mfgb_bk1_evector(9, 1, None, None, None, None, 0, None) == _abi.ERR_INVALID_ARG
    assert L.mfgb_bk3_evector(2, 1, None, None, None, None, None, 2, None) == _abi.ERR_INVALID_ARG
    assert L.mfgb_bk1_evector(2, 0, None, None, None, None, 0, None) == _abi.OK
    # tensor-core BK1: degree 1..6, mass operator only
    assert L.mfgb_bk1_evector(7, 0, None, None, None, None, 3, None) == _abi.ERR_UNSUPPORTED
    assert L.mfgb_bk3_evector(2, 0, None, None, None, None, None, 3, None) == _abi.ERR_UNSUPPORTED
    assert L.mfgb_bk1_evector(2, 0, None, None, None, None, 3, None) == _abi.OK
