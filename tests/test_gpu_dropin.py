"""Runs the C++ port of the reference's test suite (tests/cpp/test_tensor.cu)
against the drop-in tensor.cuh + libgbla.so on the GPU."""
import os
import subprocess

import pytest

from gputils_gb300 import build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin_binary(gbla_lib):
    out = os.path.join(ROOT, "_build", "test_tensor_dropin")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    cmd = [build.nvcc(), "-std=c++20", "-O1", *build.ARCH, "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "tests", "cpp"), f'-DGOLDEN_DIR="{os.path.join(ROOT, "tests", "golden")}"',
           os.path.join(ROOT, "tests", "cpp", "test_tensor.cu"), "-L", os.path.dirname(build.LIB), "-lgbla",
           "-Xlinker", f"-rpath,{os.path.dirname(build.LIB)}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


def test_reference_suite_on_dropin_header(dropin_binary, tmp_path):
    r = subprocess.run([dropin_binary], capture_output=True, text=True, cwd=tmp_path, timeout=600)
    print(r.stdout[-6000:])
    assert "0 failed" in r.stdout and r.returncode == 0, r.stdout[-6000:] + r.stderr[-2000:]
