"""Arithmetic-pipe throughput of the running GPU (mfgb_pipe_rate): FP64 FMA,
FP32 FMA, FP64 tensor-core MMA (m8n8k4), BF16 tensor-core mma.sync and the
packed dual FP32 FMA (fma.rn.f32x2), alone and interleaved with one integer
logic instruction per FMA step, in FLOP/s.  These rates decide the operator kernels' arithmetic: FP64-accurate
applies run as float pairs on the FP32 pipes because the FP64 pipes, scalar
and tensor, are far slower on this part.

    python -m benchmarks_gb300.rates [--iters 4096] [--reps 5]
    python -m benchmarks_gb300.rates --link    # host link, GB/s
"""
from __future__ import annotations

import argparse
import ctypes
import json

from . import _abi
from ._abi import lib

PIPES = {"fp64_fma": 0, "fp32_fma": 1, "fp64_mma_m8n8k4": 2, "bf16_mma_m16n8k16": 3,
         "fp32x2_fma": 4, "fp32_fma_with_lop3": 5, "fp32x2_fma_with_lop3": 6}


def pipe_rates(iters=4096, reps=5):
    out = {}
    for name, code in PIPES.items():
        r = ctypes.c_double()
        _abi.check(lib().mfgb_pipe_rate(code, iters, reps, ctypes.byref(r)))
        out[name] = r.value
    return out


LINKS = {"h2d": 0, "d2h": 1, "both": 2, "sm_h2d": 3, "sm_d2h": 4, "sm_both": 5}


def link_rates(nbytes=1 << 29, reps=3, modes=("h2d", "d2h", "both")):
    """Host link throughput in bytes/s (both directions summed for "both"),
    pinned host buffers of nbytes (mfgb_link_rate)."""
    out = {}
    for name in modes:
        r = ctypes.c_double()
        _abi.check(lib().mfgb_link_rate(LINKS[name], int(nbytes) // 16 * 16, reps, ctypes.byref(r)))
        out[name] = r.value
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m benchmarks_gb300.rates")
    ap.add_argument("--iters", type=int, default=4096)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--link", action="store_true",
                    help="host link throughput (copy engines and SM copies) instead")
    a = ap.parse_args(argv)
    if a.link:
        r = link_rates(modes=tuple(LINKS))
        print(json.dumps({k: v / 1e9 for k, v in r.items()} | {"unit": "GB/s"}))
        return
    r = pipe_rates(a.iters, a.reps)
    print(json.dumps({k: v / 1e12 for k, v in r.items()} | {"unit": "TFLOP/s"}))


if __name__ == "__main__":
    main()
