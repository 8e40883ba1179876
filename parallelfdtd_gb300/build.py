"""Build recipe for libpfdtd.so (CUDA kernels, C ABI and the C++ host API).

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a) with -lineinfo; host C++ files are
compiled with -ffp-contract=off because they evaluate update coefficients that
must round exactly as the reference source does.  Objects are compiled in
parallel and linked into parallelfdtd_gb300/libpfdtd.so (in-tree, git-ignored).
Portable flags only: the same recipe runs on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpfdtd.so")

CUDA_SOURCES = ["stencil.cu", "stencil_tma.cu", "stencil_tb.cu", "stencil_tb_f32.cu",
                "stencil_tb_f16.cu", "stencil_tb_bf16.cu", "dif.cu", "domain.cu", "setup.cu",
                "noalloc.cu", "voxelize.cu", "postfilter.cu"]
CXX_SOURCES = [
    "classes_host.cpp",
    "host/logger.cpp",
    "host/SrcRec.cpp",
    "host/SimulationParameters.cpp",
    "host/MaterialHandler.cpp",
    "host/CudaMesh.cpp",
    "host/kernels3d.cpp",
    "host/App.cpp",
    "host/app_capi.cpp",
    "host/server.cpp",
]
HEADERS_DIRS = [CSRC, os.path.join(CSRC, "host"), INCLUDE, os.path.join(INCLUDE, "pfdtd")]

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

# The blocked-update units hold only explicitly rounded arithmetic and integer
# indexing; -fmad=false states that no contraction is wanted there.
TB_SOURCES = ("stencil_tb_f32.cu", "stencil_tb_f16.cu", "stencil_tb_bf16.cu")


def _extra_flags(src: str):
    return ["-fmad=false"] if os.path.basename(src) in TB_SOURCES else []


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(_nvcc()))


def _sources():
    return ([os.path.join(CSRC, s) for s in CUDA_SOURCES],
            [os.path.join(CSRC, s) for s in CXX_SOURCES if os.path.exists(os.path.join(CSRC, s))])


def _newest_input() -> float:
    t = 0.0
    for d in HEADERS_DIRS:
        if os.path.isdir(d):
            for f in os.listdir(d):
                if f.endswith((".h", ".cuh", ".cu", ".cpp")):
                    t = max(t, os.path.getmtime(os.path.join(d, f)))
    return max(t, os.path.getmtime(__file__))


def _obj(src: str) -> str:
    rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
    return os.path.join(BUILD, rel + ".o")


def _compile(src: str, cuda: bool) -> str:
    obj = _obj(src)
    inc = ["-I" + INCLUDE, "-I" + os.path.join(INCLUDE, "pfdtd"), "-I" + CSRC,
           "-I" + os.path.join(_cuda_home(), "include")]
    if cuda:
        cmd = [_nvcc(), *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v" if os.environ.get("PFDTD_PTXAS_V") else "-O3",
               *_extra_flags(src), *inc, "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               *inc, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if os.environ.get("PFDTD_PTXAS_V") and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link libpfdtd.so; returns its path."""
    cu, cxx = _sources()
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    jobs = [(s, True) for s in cu] + [(s, False) for s in cxx]
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *GENCODE, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
