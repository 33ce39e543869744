"""Per-degree kernel-shape autotuner (no counterpart in the reference, whose
launch shape is a compile-time choice: CEED_BK/src/BK5/templated_cuda_benchmark.cc:114-124).

For each (arithmetic, degree) it times every thread layout the library has
(0 column, 1 point-per-thread, 2 column with bulk-TMA prefetch, 3 and 4 the
column and bulk-TMA kernels at an alternative number of cells per thread block,
i.e. the elements-per-block choice; for double-float also 5 and 6, the
offset-accumulation kernel at the shape-2 and shape-4 cells per block) on a
representative deformed box mesh with CUDA events, and installs the fastest in
the library's shape table (``mfgb_set_kernel_shape``).  Results can be saved
to and loaded from a small JSON file.
"""
from __future__ import annotations

import ctypes
import json

from . import _abi
from ._abi import lib

ARITHS = {"fp64": 0, "df": 1, "fp32": 2}
SHAPES = (0, 1, 2, 3, 4)
DF_SHAPES = SHAPES + (5, 6)  # double-float: the offset-accumulation kernel as well


def shapes_for(arith: int):
    return DF_SHAPES if arith == ARITHS["df"] else SHAPES


def _mesh_for(degree, target_dofs):
    import benchmarks_gb300 as mf
    n = max(2, round((target_dofs ** (1.0 / 3.0) - 1) / degree))
    return mf.BoxMesh(n, n, n, degree=degree, amplitude=0.05)


def time_shape(A, arith, shape, reps=10):
    """Milliseconds per operator application with the given shape."""
    import torch
    L = lib()
    degree = A.degree
    old = ctypes.c_int()
    _abi.check(L.mfgb_get_kernel_shape(arith, degree, ctypes.byref(old)))
    _abi.check(L.mfgb_set_kernel_shape(arith, degree, shape))
    try:
        n = A.m()
        dt = torch.float32 if arith == 2 else torch.float64
        src = torch.rand(n, dtype=dt, device="cuda")
        dst = torch.zeros_like(src)
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def once():
            if arith == 2:
                _abi.check(L.mfgb_vmult_f32(A.handle, ctypes.c_void_p(dst.data_ptr()),
                                            ctypes.c_void_p(src.data_ptr()), sp))
            else:
                _abi.check(L.mfgb_vmult(A.handle, ctypes.c_void_p(dst.data_ptr()),
                                        ctypes.c_void_p(src.data_ptr()), arith, sp))
        for _ in range(3):
            once()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            once()
        e1.record()
        torch.cuda.synchronize()
        _abi.check(L.mfgb_check_device_errors(sp))  # a timed-out kernel is not a result
        return e0.elapsed_time(e1) / reps
    finally:
        _abi.check(L.mfgb_set_kernel_shape(arith, degree, old.value))


def tune(degrees=range(1, 9), ariths=("df", "fp32"), target_dofs=2.0e7, reps=10, apply=True):
    """Times every shape; returns {arith: {degree: {"best": s, "ms": [..]}}} and
    (with apply) installs the winners."""
    import benchmarks_gb300 as mf
    result = {}
    for d in degrees:
        A = mf.LaplaceOperator(_mesh_for(d, target_dofs))
        for name in ariths:
            a = ARITHS[name]
            shapes = shapes_for(a)
            ms = [time_shape(A, a, s, reps) for s in shapes]
            best = min(range(len(shapes)), key=lambda i: ms[i])
            result.setdefault(name, {})[d] = {"best": shapes[best], "ms": ms, "n_dofs": A.m(),
                                              "shapes": list(shapes)}
            if apply:
                _abi.check(lib().mfgb_set_kernel_shape(a, d, shapes[best]))
        del A
    return result


def save(result, path):
    with open(path, "w") as f:
        json.dump(result, f, indent=1)


def load(path, apply=True):
    with open(path) as f:
        result = json.load(f)
    if apply:
        for name, per in result.items():
            for d, r in per.items():
                _abi.check(lib().mfgb_set_kernel_shape(ARITHS[name], int(d), int(r["best"])))
    return result


def main(argv=None):
    """Command line: re-measure the shape table, or time one shape (for profiling).

    python -m benchmarks_gb300.autotune [--degrees 1 2 ...] [--ariths df fp32 fp64]
        [--dofs 3e7] [--reps 10] [--shape S] [--out table.json]
    """
    import argparse
    ap = argparse.ArgumentParser(prog="python -m benchmarks_gb300.autotune")
    ap.add_argument("--degrees", type=int, nargs="+", default=list(range(1, 9)))
    ap.add_argument("--ariths", nargs="+", choices=sorted(ARITHS), default=["df", "fp32"])
    ap.add_argument("--dofs", type=float, default=2.0e7, help="DoFs of the timing mesh")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--shape", type=int, choices=DF_SHAPES, default=None,
                    help="time only this shape (no tuning)")
    ap.add_argument("--out", default=None, help="write the measured table as JSON")
    a = ap.parse_args(argv)
    import torch

    import benchmarks_gb300 as mf
    torch.cuda.set_device(0)
    if a.shape is not None:
        for d in a.degrees:
            A = mf.LaplaceOperator(_mesh_for(d, a.dofs))
            for name in a.ariths:
                ms = time_shape(A, ARITHS[name], a.shape, a.reps)
                print(json.dumps({"arith": name, "degree": d, "shape": a.shape, "n_dofs": A.m(),
                                  "ms": ms, "GDoF/s": A.m() / ms / 1e6}))
            del A
        return
    r = tune(a.degrees, tuple(a.ariths), a.dofs, a.reps, apply=True)
    print(json.dumps(r))
    if a.out:
        save(r, a.out)


if __name__ == "__main__":
    main()
