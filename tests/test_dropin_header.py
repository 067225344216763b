"""The drop-in tensor.cuh has no device code: it must compile as plain C++
(C++17 and C++20) together with the C++ port of the reference's tests."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


@pytest.mark.parametrize("std", ["c++17", "c++20"])
def test_header_compiles_as_plain_cpp(std):
    cmd = ["g++", f"-std={std}", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           _cuda_include(), "-I", os.path.join(ROOT, "tests", "cpp"), '-DGOLDEN_DIR="tests/golden"', "-x", "c++",
           os.path.join(ROOT, "tests", "cpp", "test_tensor.cu")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
