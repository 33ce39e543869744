"""Host-side pieces of the batched solver (no GPU needed)."""
import benchmarks_gb300 as mf


def test_workload_generator_is_seeded():
    a, sa = mf.batch_workload(16, seed=5)
    b, sb = mf.batch_workload(16, seed=5)
    assert a == b and sa == sb
    assert all(2 <= m.degree <= 7 and 6 <= m.nx <= 32 and m.nx == m.ny == m.nz and
               0 <= m.amplitude <= 0.1 for m in a)
    c, _ = mf.batch_workload(16, seed=6)
    assert a != c


def test_workload_size_of_the_256_problem_mix():
    meshes, seeds = mf.batch_workload(256, seed=2024)
    total = sum(m.n_dofs for m in meshes)
    assert len(set(seeds)) == 256
    assert 1.0e8 < total < 8.0e8  # about 3.4e8 DoFs expected for this mix


def test_sweep_meshes_hit_the_target_sizes():
    """The degree x size sweep's meshes (n^3 cells, n = round((N^(1/3) - 1)/p))
    stay within a factor 1.6 of every target size for p = 1..8."""
    from benchmarks_gb300 import sweep
    for p in range(1, 9):
        for target in (1e5, 1e6, 1e7, 1.5e8):
            mesh, n = sweep._mesh(mf, p, target)
            assert mesh.nx == mesh.ny == mesh.nz == n and mesh.degree == p
            assert target / 1.6 <= mesh.n_dofs <= target * 1.6
