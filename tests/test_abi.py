"""The C ABI library loads and exports every entry point include/mfgb.h declares
(no compute call: runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(mfgb_\w+)\s*\(", text, re.M))
    return sorted(names)


@pytest.fixture(scope="module")
def libmfgb():
    from benchmarks_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for need in ("mfgb_vmult", "mfgb_bk5_lvector", "mfgb_bk5_evector", "mfgb_cg_solve",
                 "mfgb_compute_diagonal", "mfgb_operator_create_box"):
        assert need in syms


def test_library_exports_every_declared_symbol(libmfgb):
    missing = [s for s in declared_symbols() if not hasattr(libmfgb, s)]
    assert not missing, missing


def test_status_strings(libmfgb):
    libmfgb.mfgb_status_string.restype = ctypes.c_char_p
    assert libmfgb.mfgb_status_string(0) == b"ok"
    assert libmfgb.mfgb_status_string(2) == b"out of device memory"
    libmfgb.mfgb_version.restype = ctypes.c_int
    assert libmfgb.mfgb_version() >= 1


def test_invalid_arguments_are_rejected_without_gpu(libmfgb):
    """Argument validation happens before any CUDA call."""
    import benchmarks_gb300 as mf
    from benchmarks_gb300 import _abi
    L = mf.lib()
    op = ctypes.c_void_p()
    bad = _abi.BoxDesc(2, 2, 2, 9, (ctypes.c_double * 3)(0, 0, 0), (ctypes.c_double * 3)(1, 1, 1), 0.0)
    assert L.mfgb_operator_create_box(ctypes.byref(bad), ctypes.byref(op)) == _abi.ERR_INVALID_ARG
    assert b"degree" in L.mfgb_last_error()
    assert L.mfgb_bk5_evector(0, 1, None, None, None, None, 0, None) == _abi.ERR_INVALID_ARG
    assert L.mfgb_vmult(None, None, None, 0, None) == _abi.ERR_INVALID_ARG
    assert L.mfgb_cg_solve(None, None, None, None, None, None, None) == _abi.ERR_INVALID_ARG
    with pytest.raises(ValueError):
        mf._arith("fp16")


def test_kernel_shape_table_round_trip_without_gpu(libmfgb):
    """The autotuner's shape table (thread layout and cells per CTA per degree):
    every shape the autotuner times is accepted, others are rejected, and the
    defaults come back after a round trip.  Host-only calls."""
    import benchmarks_gb300 as mf
    from benchmarks_gb300 import _abi, autotune
    L = mf.lib()
    assert tuple(autotune.SHAPES) == (0, 1, 2, 3, 4)
    assert tuple(autotune.shapes_for(1)) == (0, 1, 2, 3, 4, 5, 6)  # + offset accumulation
    for arith in autotune.ARITHS.values():
        for degree in range(1, 9):
            old = ctypes.c_int()
            assert L.mfgb_get_kernel_shape(arith, degree, ctypes.byref(old)) == _abi.OK
            assert old.value in autotune.shapes_for(arith)
            for shape in autotune.shapes_for(arith):
                assert L.mfgb_set_kernel_shape(arith, degree, shape) == _abi.OK
                got = ctypes.c_int()
                assert L.mfgb_get_kernel_shape(arith, degree, ctypes.byref(got)) == _abi.OK
                assert got.value == shape
            assert L.mfgb_set_kernel_shape(arith, degree, old.value) == _abi.OK
    assert L.mfgb_set_kernel_shape(1, 4, 7) == _abi.ERR_INVALID_ARG
    assert L.mfgb_set_kernel_shape(0, 4, 5) == _abi.ERR_INVALID_ARG  # double-float only
    assert L.mfgb_set_kernel_shape(2, 4, 5) == _abi.ERR_INVALID_ARG
    assert L.mfgb_set_kernel_shape(1, 9, 0) == _abi.ERR_INVALID_ARG
    assert L.mfgb_set_kernel_shape(3, 4, 0) == _abi.ERR_INVALID_ARG
    assert L.mfgb_set_host_pipeline(65) == _abi.ERR_INVALID_ARG
    assert L.mfgb_set_host_pipeline(0) == _abi.OK  # automatic slab count
