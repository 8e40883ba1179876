"""The reference's CudaMesh device tests (element indexing, partition
get/set and halos, 1/2/5-partition invariance in float and double, an App
run) restated in C++ against this library's C++ API."""
import subprocess

import pytest

from test_host_api_cpp import compile_cpp

pytestmark = pytest.mark.gpu


def test_cudamesh_cpp(gpu, tmp_path):
    exe = compile_cpp("cudamesh_test.cpp", str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout, r.stderr[-2000:])
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
