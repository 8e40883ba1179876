"""Compile the reference's MATLAB gateway (matlab/mex_FDTD.cpp, read where it
lies in the reference tree) against this library's drop-in headers and the
stand-in MEX API of this folder, and link it with libpfdtd.so.

    python tests/mex_stub/build_gateway.py <out_dir> [reference_dir]

reference_dir defaults to where the oracle's reference build recipe finds the
reference (oracle/build_ref.py: $PFDTD_REFERENCE_DIR, else its mount point);
None when it is absent.  Prints the path of the linked host program.  Nothing
is copied out of the reference.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def reference_dir(arg: str | None = None) -> str | None:
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    from oracle import build_ref
    return build_ref.reference_dir(arg)


def gateway_source(ref: str) -> str:
    return os.path.join(ref, "matlab", "mex_FDTD.cpp")


def build(out_dir: str, ref: str | None = None) -> str:
    where = reference_dir(ref)
    if where is None:
        raise FileNotFoundError("reference sources not found (set PFDTD_REFERENCE_DIR)")
    src = gateway_source(where)
    lib_dir = os.path.join(REPO, "parallelfdtd_gb300")
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    inc = ["-I" + HERE, "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(REPO, "include", "pfdtd"), "-I" + cuda_inc]
    os.makedirs(out_dir, exist_ok=True)
    gw = os.path.join(out_dir, "mex_FDTD.o")
    host = os.path.join(out_dir, "mex_host.o")
    exe = os.path.join(out_dir, "mex_host")
    subprocess.run(["g++", "-std=c++17", "-O1", *inc, "-c", src, "-o", gw], check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + HERE, "-c",
                    os.path.join(HERE, "mex_host.cpp"), "-o", host], check=True)
    subprocess.run(["g++", gw, host, "-L" + lib_dir, "-lpfdtd", "-Wl,-rpath," + lib_dir,
                    "-o", exe], check=True)
    return exe


if __name__ == "__main__":
    print(build(sys.argv[1], sys.argv[2] if len(sys.argv) > 2 else None))
