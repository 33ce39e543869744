"""Host-side pieces of bench.py (no GPU): the algorithmic byte and flop counts
behind `roofline`, the DRAM traffic read from the committed ncu summary, the
peak denominator and the workload description."""
import argparse
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    import sys
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench as b
    return b


def test_algorithmic_bytes_per_dof(bench):
    """8N + 8N + n_c (p+1)^3 (48 + 4): 432, 192, 139, 118, 106, 99, 94, 90 B/DoF
    for p = 1..8 on large meshes."""
    want = {1: 432, 2: 192, 3: 139, 4: 118, 5: 106, 6: 99, 7: 94, 8: 90}
    for p, bpd in want.items():
        n = 400 // p
        n_dofs = (p * n + 1) ** 3
        got = bench.algorithmic_bytes(n_dofs, n ** 3, p) / n_dofs
        assert abs(got - bpd) < 0.02 * bpd, (p, got)


def test_algorithmic_flops(bench):
    assert bench.algorithmic_flops(1, 4) == 12 * 5 ** 4 + 15 * 5 ** 3


def test_traffic_from_the_committed_profile(bench):
    """The bench line's `traffic` is the DRAM bytes per launch recorded in
    profiles/bk5_df_p4_67M.md for the headline workload (None elsewhere)."""
    saved = dict(bench.WORKLOAD)
    try:
        t = bench.traffic_from_profile("df")
        assert t is not None and 5e9 < t < 2e10
        algo = bench.algorithmic_bytes(67634433, 128 * 128 * 64, 4)
        assert 1.0 <= t / algo < 1.3  # no large re-reads
        bench.WORKLOAD.update(nx=64)
        assert bench.traffic_from_profile("df") is None
    finally:
        bench.WORKLOAD.clear()
        bench.WORKLOAD.update(saved)


def test_peak_denominator(bench):
    peak, kind = bench.measured_peaks()
    assert peak > 1000 and kind in ("measured", "fallback")


def test_workload_config(bench):
    args = argparse.Namespace(arith="df", shape="auto", gpus=1)
    c = bench.config_dict(args, 67634433, 128 * 128 * 64)
    assert c["n_dofs"] == 67634433 and c["degree"] == 4 and c["cells"] == [128, 128, 64]
    assert "workload" in c and bench.is_headline()
