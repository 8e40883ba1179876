"""C++ host classes with the reference's names (SimulationParameters,
MaterialHandler, CudaMesh partition indexing), checked by a C++ program that
restates the reference's own unit tests.  Needs no GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_cpp(name: str, out_dir: str) -> str:
    from parallelfdtd_gb300 import _lib
    src = os.path.join(ROOT, "tests", "cpp", name)
    exe = os.path.join(out_dir, name.replace(".cpp", ""))
    pkg = os.path.dirname(_lib.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "include", "pfdtd"), "-I/usr/local/cuda/include",
           src, "-o", exe, "-L" + pkg, "-lpfdtd", "-Wl,-rpath," + pkg,
           "-L/usr/local/cuda/lib64", "-lcudart"]
    subprocess.check_call(cmd)
    return exe


def test_host_api(built, tmp_path):
    exe = compile_cpp("host_api_test.cpp", str(tmp_path))
    ir = os.path.join(ROOT, "tests", "golden", "grid_ir_kat.txt")
    r = subprocess.run([exe, ir], capture_output=True, text=True)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout


def test_host_classes_equal_reference_golden(built, tmp_path):
    """Source samples of every source and input type (float and double),
    parameter vectors and a material table with repeated materials: this
    library's classes against the values the reference's own classes gave
    (tests/golden/ref_host_golden.txt, made by tests/golden/make_ref_golden.py)."""
    exe = compile_cpp("golden_host_test.cpp", str(tmp_path))
    gold = os.path.join(ROOT, "tests", "golden", "ref_host_golden.txt")
    ir = os.path.join(ROOT, "tests", "golden", "grid_ir_kat.txt")
    r = subprocess.run([exe, gold, ir], capture_output=True, text=True, cwd=str(tmp_path))
    print(r.stdout[-3000:])
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    assert " 0 failures" in r.stdout
