"""The header-only C++ adapter (include/mfgb_operator.hpp) compiles with every
member of its operator classes instantiated (g++ -fsyntax-only against the CUDA
runtime headers; no GPU, no link).  The GPU test runs the example program."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SOURCE = r"""
#include "mfgb_operator.hpp"
template class mfgb::LaplaceOperatorBK35<3, 4, double>;
template class mfgb::HelmholtzOperator<3, 4, double>;
template class mfgb::LaplaceOperatorBP3<3, 4, double>;
int main() { return 0; }
"""


def cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_adapter_instantiates(tmp_path):
    cxx = shutil.which("g++")
    inc = cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA runtime headers")
    src = tmp_path / "adapter.cc"
    src.write_text(SOURCE)
    out = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                          "-I", inc, str(src)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
