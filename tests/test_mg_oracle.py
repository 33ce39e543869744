"""CPU checks of the multigrid oracle's level construction and transfers
(coarsening of any cell count: level l keeps the fine nodes min(k 2^l, n))."""
import numpy as np
import pytest

from oracle import mg_oracle
from oracle import oracle as orc


@pytest.mark.parametrize("nf,s", [(8, 1), (7, 1), (7, 2), (31, 4), (27, 8), (6, 2)])
def test_h_matrix_reproduces_linear_functions(nf, s):
    P = mg_oracle.MGOracle._h_matrix_1d(nf, s)
    m, mc = P.shape[0] - 1, P.shape[1] - 1
    assert m == -(-nf // s) and mc == -(-nf // (2 * s))
    xf = np.minimum(np.arange(m + 1) * s, nf) / nf
    xc = np.minimum(np.arange(mc + 1) * 2 * s, nf) / nf
    for f in (np.ones_like, lambda x: 3 * x - 1):
        assert np.allclose(P @ f(xc), f(xf), rtol=0, atol=1e-15)
    assert np.all(P >= 0) and np.allclose(P.sum(1), 1.0)


def test_stride_one_box_is_the_uniform_box():
    a = orc.BoxProblem(3, 4, 5, 2, amplitude=0.1)
    b = orc.BoxProblem(3, 4, 5, 2, amplitude=0.1, stride=1, nf=(3, 4, 5))
    assert np.array_equal(a.G, b.G)


@pytest.mark.parametrize("nf,s", [(7, 2), (9, 4), (5, 2)])
def test_coarse_cells_are_unions_of_fine_cells(nf, s):
    """Cell corners of the strided level sit on fine mesh nodes."""
    nc = -(-nf // s)
    C = orc.BoxProblem(nc, nc, nc, 1, amplitude=0.0, stride=s, nf=(nf, nf, nf), geometry_degree=1)
    for cell in range(C.n_cells):
        cx, cy, cz = cell % nc, (cell // nc) % nc, cell // (nc * nc)
        xyz = C.cell_nodes(cell).reshape(2, 2, 2, 3)
        for d, c in enumerate((cx, cy, cz)):
            lo, hi = min(c * s, nf) / nf, min((c + 1) * s, nf) / nf
            # node index order (i, j, k) = (z, y, x)
            ax = {0: (slice(None), slice(None), 0), 1: (slice(None), 0, slice(None)),
                  2: (0, slice(None), slice(None))}[d]
            assert np.allclose(xyz[ax][..., d], lo, atol=1e-15)
    with pytest.raises(ValueError):
        orc.BoxProblem(nc + 1, nc, nc, 1, stride=s, nf=(nf, nf, nf))


def test_odd_mesh_hierarchy():
    M = mg_oracle.MGOracle(7, 7, 5, 2, amplitude=0.05, eig_iterations=3, coarse_cells=2)
    assert [L.degree for L in M.levels] == [2, 1, 1, 1]
    assert [L.box for L in M.levels] == [(7, 7, 5), (7, 7, 5), (4, 4, 3), (2, 2, 2)]
    assert [L.stride for L in M.levels] == [1, 1, 2, 4]
    assert M.coarse_A.shape == (1, 1)
