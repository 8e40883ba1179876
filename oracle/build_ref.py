"""Build recipe for oracle/_ref: the reference's own code, compiled from its
unchanged sources where they lie — test infrastructure only.

ParallelFDTD as a whole does not build here (Boost.Python, GL, the external
voxelizer; its CMake gencodes predate nvcc 13), but the files on the hot path
do.  This recipe compiles them without the reference's build system and
writes only into oracle/_ref/ (git-ignored):

1. libref_cpu.so (host, for golden vectors made in this container):
   - src/base/SimulationParameters.cpp, MaterialHandler.cpp, SrcRec.cpp and
     what SimulationParameters::readGridIr links to (src/io/FileReader.cpp,
     src/base/GeometryHandler.cpp), unchanged, with a stand-in for
     <boost/format.hpp> (oracle/ref_stub/);
   - the kernels fdtd3dStdMaterials and fdtd3dStdKowalczykMaterials
     (src/kernels/kernels3d.cu) and the node-translation, counting and padding
     kernels toBilbao/toKowalczyk/toBilbaoKernel/toKowalczykKernel/
     calcBoundaries/padWithZerosKernel (src/kernels/cudaMesh.cu), their text
     taken unchanged from those files and compiled as host C++ behind the
     prelude oracle/ref_cpu_emul.h and the launch loops
     oracle/ref_cpu_launch.inc.  The text is piped to g++ on stdin; no copy
     of it is written to disk;
   - oracle/ref_host_capi.cpp, a C interface to the classes above.
2. kernels3d_sm103a.cubin, kernels3d_sm103a_nofma.cubin,
   cudaMesh_sm103a.cubin: src/kernels/kernels3d.cu and cudaMesh.cu compiled
   unchanged by nvcc for sm_103a, device code only, with nvcc's default
   floating-point contraction and with -fmad=false.  A cubin is GPU code and
   runs on any host architecture; oracle/ref_gpu_runner.cpp (built on the GPU
   machine by oracle/build.py) loads it with the CUDA driver API.

The reference location comes from PFDTD_REFERENCE_DIR or --reference; the
default is where this container mounts it.  Where the reference is absent
(for instance on a machine that only receives the built files) build() does
nothing and returns False.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
STUB = os.path.join(HERE, "ref_stub")
LIB = os.path.join(OUT, "libref_cpu.so")
CUBINS = {
    "kernels3d": os.path.join(OUT, "kernels3d_sm103a.cubin"),
    "kernels3d_nofma": os.path.join(OUT, "kernels3d_sm103a_nofma.cubin"),
    "cudaMesh": os.path.join(OUT, "cudaMesh_sm103a.cubin"),
}
DEFAULT_REFERENCE = "/root/reference"

HOST_SOURCES = ["src/base/SimulationParameters.cpp", "src/base/MaterialHandler.cpp",
                "src/base/SrcRec.cpp", "src/io/FileReader.cpp", "src/base/GeometryHandler.cpp"]
# (file, function names) whose definitions are compiled for the host
KERNEL_TEXT = [
    ("src/kernels/cudaMesh.cu", ["toBilbao", "toKowalczyk", "toKowalczykKernel",
                                 "toBilbaoKernel", "calcBoundaries", "padWithZerosKernel"]),
    ("src/kernels/kernels3d.cu", ["fdtd3dStdMaterials", "fdtd3dStdKowalczykMaterials"]),
]
MASK_HEADER = "src/kernels/cudaMesh.h"
MASK_NAMES = ["INSIDE_SWITCH", "FORWARD_POSITION_MASK", "CENTERED_MASK", "DIR_X", "DIR_Y",
              "DIR_Z", "SIGN_X", "SIGN_Y", "SIGN_Z"]


def reference_dir(explicit: str | None = None) -> str | None:
    for cand in (explicit, os.environ.get("PFDTD_REFERENCE_DIR"), DEFAULT_REFERENCE):
        if cand and os.path.isfile(os.path.join(cand, "src", "kernels", "kernels3d.cu")):
            return cand
    return None


def _definition(text: str, name: str) -> tuple[int, str]:
    """(first line number, text) of the definition of function `name`,
    including a `template <...>` line directly above it."""
    for m in re.finditer(r"\b" + re.escape(name) + r"\s*\(", text):
        # skip calls and declarations: the signature must start a line with a type
        line_start = text.rfind("\n", 0, m.start()) + 1
        head = text[line_start:m.start()]
        if "void" not in head:
            continue
        depth, i = 0, m.end() - 1
        while i < len(text):
            if text[i] == "(":
                depth += 1
            elif text[i] == ")":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        j = i + 1
        while j < len(text) and text[j].isspace():
            j += 1
        if j >= len(text) or text[j] != "{":
            continue  # a declaration
        depth, k = 0, j
        while k < len(text):
            if text[k] == "{":
                depth += 1
            elif text[k] == "}":
                depth -= 1
                if depth == 0:
                    break
            k += 1
        start = line_start
        prev_start = text.rfind("\n", 0, max(line_start - 1, 0)) + 1
        if text[prev_start:line_start].strip().startswith("template"):
            start = prev_start
        return text.count("\n", 0, start) + 1, text[start:k + 1]
    raise RuntimeError(f"definition of {name} not found")


def _kernel_unit(ref: str) -> str:
    parts = ['#include "ref_cpu_emul.h"\n']
    with open(os.path.join(ref, MASK_HEADER)) as f:
        header = f.read()
    for name in MASK_NAMES:
        m = re.search(r"^#define\s+" + name + r"\s+\S+.*$", header, re.M)
        if not m:
            raise RuntimeError(f"{name} not found in {MASK_HEADER}")
        line = header.count("\n", 0, m.start()) + 1
        parts.append(f'#line {line} "{MASK_HEADER}"\n{m.group(0)}\n')
    for rel, names in KERNEL_TEXT:
        with open(os.path.join(ref, rel)) as f:
            text = f.read()
        for name in names:
            line, body = _definition(text, name)
            parts.append(f'#line {line} "{rel}"\n{body}\n')
    parts.append('#line 1 "oracle/ref_cpu_launch.inc"\n#include "ref_cpu_launch.inc"\n')
    return "".join(parts)


def _run(cmd, stdin: str | None = None, cwd: str | None = None):
    r = subprocess.run(cmd, input=stdin, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    return None


def _inputs_newer(out: str, files) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(f) > t for f in files if os.path.exists(f))


def build(reference: str | None = None, force: bool = False) -> bool:
    ref = reference_dir(reference)
    if ref is None:
        return False
    os.makedirs(OUT, exist_ok=True)
    ours = [os.path.join(HERE, f) for f in ("ref_cpu_emul.h", "ref_cpu_launch.inc",
                                            "ref_host_capi.cpp", "build_ref.py")]
    ours.append(os.path.join(STUB, "boost", "format.hpp"))
    theirs = [os.path.join(ref, f) for f in HOST_SOURCES + [MASK_HEADER] +
              [k for k, _ in KERNEL_TEXT]]
    inc = ["-I" + STUB, "-I" + HERE]
    cuda_inc = "/usr/local/cuda/include"
    nvcc = _nvcc()
    if nvcc:
        cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    flags = ["-O2", "-std=c++14", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
             "-w"]
    if force or _inputs_newer(LIB, ours + theirs):
        objs = []
        tmp = os.path.join(OUT, "obj")
        os.makedirs(tmp, exist_ok=True)
        for rel in HOST_SOURCES:
            obj = os.path.join(tmp, os.path.basename(rel) + ".o")
            _run(["g++", *flags, *inc, "-I" + cuda_inc, "-c", os.path.join(ref, rel), "-o", obj])
            objs.append(obj)
        kobj = os.path.join(tmp, "ref_kernels_cpu.o")
        _run(["g++", *flags, *inc, "-x", "c++", "-c", "-", "-o", kobj], stdin=_kernel_unit(ref),
             cwd=ref)
        objs.append(kobj)
        capi = os.path.join(tmp, "ref_host_capi.o")
        _run(["g++", *flags, *inc, "-I" + os.path.join(ref, "src"), "-I" + cuda_inc, "-c",
              os.path.join(HERE, "ref_host_capi.cpp"), "-o", capi])
        objs.append(capi)
        _run(["g++", "-shared", "-fopenmp", "-o", LIB + ".tmp", *objs])
        os.replace(LIB + ".tmp", LIB)
    if nvcc:
        gencode = ["-gencode", "arch=compute_103a,code=sm_103a"]
        jobs = [("kernels3d", "src/kernels/kernels3d.cu", []),
                ("kernels3d_nofma", "src/kernels/kernels3d.cu", ["-fmad=false"]),
                ("cudaMesh", "src/kernels/cudaMesh.cu", [])]
        for key, rel, extra in jobs:
            out = CUBINS[key]
            if force or _inputs_newer(out, [os.path.join(ref, rel), os.path.join(ref, MASK_HEADER),
                                            os.path.join(STUB, "boost", "format.hpp")]):
                _run([nvcc, "-cubin", *gencode, "-std=c++14", "-w", *extra, "-I" + STUB,
                      os.path.join(ref, rel), "-o", out + ".tmp"])
                os.replace(out + ".tmp", out)
    return True


def cubins_present() -> bool:
    return all(os.path.exists(p) for p in CUBINS.values())


if __name__ == "__main__":
    args = sys.argv[1:]
    explicit = None
    if "--reference" in args:
        explicit = args[args.index("--reference") + 1]
    ok = build(explicit, force="--force" in args)
    print(OUT if ok else "reference sources not found: nothing built")
