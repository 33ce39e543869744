"""The header-only C++ adapter (include/mfgb_operator.hpp) used the way the
reference's scaling driver uses its operator: the example program's CG counts
equal the Python API's on the same problem."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def example():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from benchmarks_gb300 import build
    build.build()
    return build.build_example()


def run(example, *args):
    out = subprocess.run([example, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[0].split() == ["cells", "dofs", "matvec", "CG_tot_time", "CG_time/iters",
                                "cg_its", "cg_reduction"]
    cells, dofs, mv, t, ti, its, red = lines[1].split()
    return int(cells), int(dofs), float(mv), int(its), float(red)


def test_cpp_adapter_matches_python_api(example):
    import benchmarks_gb300 as mf
    cells, dofs, mv, its, red = run(example, 8, 8, 4, "jacobi", 1e-8)
    mesh = mf.BoxMesh(8, 8, 4, degree=4, amplitude=0.05)
    A = mf.LaplaceOperator(mesh)
    assert (cells, dofs) == (A.n_cells, A.m())
    b = A.rhs_uniform(1)
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(1000000, 1e-300, 1e-8)
    P = A.get_matrix_diagonal_inverse()
    mf.SolverCG(ctl).solve(A, x, b, P)
    assert its == ctl.last_step() and 0 < red < 1 and mv > 0
    # el(row, row): the diagonal entry, 1 / the inverse diagonal
    out = subprocess.run([example, "8", "8", "4", "jacobi", "1e-8"], capture_output=True, text=True,
                         timeout=600)
    el = float([l for l in out.stdout.splitlines() if l.startswith("el_mid")][0].split()[1])
    assert el == pytest.approx(1.0 / float(P.vector[A.m() // 2]), rel=1e-15)
    _, _, _, its_mg, _ = run(example, 8, 8, 4, "mg32", 1e-10)
    assert 0 < its_mg < 30


def test_cpp_adapter_helmholtz_and_host_apply(example):
    """mfgb::HelmholtzOperator (bp5_kokkos's operator) with Jacobi-PCG through the
    adapter gives the Python API's iteration count; the host-buffer apply
    equals the device apply."""
    import benchmarks_gb300 as mf
    out = subprocess.run([example, "6", "6", "4", "helmholtz", "1e-8"], capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    its = int(lines[1].split()[5])
    diff = float(lines[-1].split()[1])
    assert lines[-1].startswith("host_apply_rel_diff") and diff <= 1e-14
    H = mf.HelmholtzOperator(mf.BoxMesh(6, 6, 4, degree=4, amplitude=0.05))
    b = H.rhs_uniform(1)
    x = H.initialize_dof_vector()
    ctl = mf.ReductionControl(1000000, 1e-300, 1e-8)
    mf.SolverCG(ctl).solve(H, x, b, H.get_matrix_diagonal_inverse())
    assert its == ctl.last_step()


def test_cpp_adapter_reports_errors(example):
    out = subprocess.run([example, "0", "1", "1"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 2 and "invalid argument" in out.stderr
