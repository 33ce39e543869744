"""Arithmetic-pipe and host-link throughput entry points (mfgb_pipe_rate,
mfgb_link_rate): the rates the operator kernels' arithmetic and the host-buffer
apply's bound rest on.  Checked for sanity, not for speed: every pipe and link
mode reports a positive rate, FP32 FMAs outrun FP64 FMAs by more than 10x on
this part, and two directions at once move at least as many bytes as one."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import benchmarks_gb300 as mf
    return mf.lib()


def test_pipe_rates(L):
    from benchmarks_gb300.rates import pipe_rates
    r = pipe_rates(iters=256, reps=1)
    assert all(v > 0 for v in r.values())
    assert r["fp32_fma"] > 10 * r["fp64_fma"]


def test_link_rates(L):
    from benchmarks_gb300.rates import link_rates, LINKS
    r = link_rates(nbytes=32 << 20, reps=1, modes=tuple(LINKS))
    assert all(v > 1e9 for v in r.values())
    assert r["both"] >= 0.9 * max(r["h2d"], r["d2h"])


def test_rate_arguments(L):
    from benchmarks_gb300 import _abi
    out = ctypes.c_double()
    assert L.mfgb_pipe_rate(7, 1, 1, ctypes.byref(out)) == _abi.ERR_INVALID_ARG
    assert L.mfgb_link_rate(6, 1 << 20, 1, ctypes.byref(out)) == _abi.ERR_INVALID_ARG
    assert L.mfgb_link_rate(0, 24, 1, ctypes.byref(out)) == _abi.ERR_INVALID_ARG
