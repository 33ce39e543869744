"""Build libmfgb.so in-tree: every CUDA translation unit compiled for sm_103a in
parallel with nvcc, then linked as one shared library (no cmake, no torch
extension machinery; the C ABI has no torch types)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmfgb.so")

SOURCES = [
    "mfgb_api.cu",
    "mfgb_setup.cu",
    "mfgb_cg.cu",
    "mfgb_mg.cu",
    "mfgb_batch.cu",
    "mfgb_bkq.cu",
    "mfgb_bp3_fx.cu",
    "mfgb_helmholtz_fx.cu",
    "mfgb_bk1_dmma.cu",
    "mfgb_bk5_f64.cu",
    "mfgb_bk5_df.cu",
    "mfgb_bk5_fx.cu",
    "mfgb_bk5_f32.cu",
    "mfgb_bk5g.cu",
    "mfgb_bk6.cu",
    "mfgb_mlp.cu",
    "mfgb_rates.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmfgb.so")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, *extra]


def _compile(src: str, extra) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "mfgb.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *_flags(extra), "-c", srcp, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


EXAMPLE = os.path.join(BUILD, "bp5_solve")


def build_example() -> str:
    """Compile the C++ example driver (header-only adapter over the C ABI)."""
    src = os.path.join(HERE, "examples", "bp5_solve.cc")
    hdrs = [os.path.join(ROOT, "include", h) for h in ("mfgb.h", "mfgb_operator.hpp")]
    if os.path.exists(EXAMPLE) and all(os.path.getmtime(EXAMPLE) >= os.path.getmtime(d)
                                       for d in [src, LIB, *hdrs]):
        return EXAMPLE
    cuda = os.path.dirname(os.path.dirname(nvcc()))
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(cuda, "include"), src, "-o", EXAMPLE, "-L" + HERE, "-lmfgb",
           "-L" + os.path.join(cuda, "lib64"), "-lcudart", "-Wl,-rpath," + HERE,
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"example build failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return EXAMPLE


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


def build_all(verbose: bool = False) -> str:
    lib = build(verbose)
    build_example()
    return lib


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
