"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/fdtd_oracle.cpp into oracle/_build/liboracle.so with
-ffp-contract=off (every product rounded before it is summed, as the reference
source is written) and OpenMP for the timed CPU baseline.  Also compiles
oracle/ref_gpu_runner.cpp into oracle/_build/libref_gpu.so, the driver-API host
loop that runs the reference's own kernels from the cubins oracle/build_ref.py
makes, and — where the reference sources are present — runs that recipe.
Portable flags only: the same recipe runs on x86_64 and aarch64.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fdtd_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
REF_GPU_SRC = os.path.join(HERE, "ref_gpu_runner.cpp")
REF_GPU_LIB = os.path.join(OUT_DIR, "libref_gpu.so")


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda.h")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    return None


def build_ref_gpu(force: bool = False):
    """libref_gpu.so (links the CUDA driver library); None without a CUDA toolkit."""
    cuda = _cuda_home()
    if cuda is None:
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(REF_GPU_LIB)
            and os.path.getmtime(REF_GPU_LIB) >= os.path.getmtime(REF_GPU_SRC)):
        return REF_GPU_LIB
    libdirs = [d for d in (os.path.join(cuda, "lib64", "stubs"), os.path.join(cuda, "lib64"),
                           os.path.join(cuda, "targets", "sbsa-linux", "lib", "stubs"))
               if os.path.isdir(d)]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", REF_GPU_SRC,
           "-I" + os.path.join(cuda, "include"), *["-L" + d for d in libdirs], "-lcuda",
           "-o", REF_GPU_LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(REF_GPU_LIB + ".tmp", REF_GPU_LIB)
    return REF_GPU_LIB


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
               "-fno-fast-math", "-fopenmp", SRC, "-o", LIB + ".tmp"]
        subprocess.check_call(cmd)
        os.replace(LIB + ".tmp", LIB)
    build_ref_gpu(force)
    # The reference's own sources exist only where they are mounted; elsewhere
    # the files this recipe made earlier (cubins) are used as they are.
    from oracle import build_ref
    build_ref.build(force=force)
    return LIB


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    print(build(force="--force" in sys.argv))
