"""The C ABI library loads and exports every function its headers declare
(no compute calls: runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("pfdtd.h", "pfdtd_app.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(pfdtd_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_functions():
    names = declared_functions()
    assert "pfdtd_run" in names and "pfdtd_app_run_simulation" in names
    assert len(names) > 60


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_every_declared_symbol(lib):
    from parallelfdtd_gb300 import _lib
    bound = set(_lib.exported_names())
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, f"declared but not bound in _lib: {missing}"


def test_reference_cpp_api_symbols_exported(built):
    """The C++ entry points with the reference's names are in the library."""
    from parallelfdtd_gb300 import _lib
    syms = os.popen(f"nm -DC {_lib.LIB_PATH}").read()
    for sym in ("launchFDTD3d(CudaMesh*, SimulationParameters*, float*",
                "launchFDTD3dDouble(CudaMesh*, SimulationParameters*, double*",
                "launchFDTD3dStep(CudaMesh*, SimulationParameters*, float*",
                "CudaMesh::setupMesh(", "CudaMesh::makePartition(",
                "FDTD::App::runSimulation()", "MaterialHandler::getMaterialCoefficientPtr()",
                "SimulationParameters::getSourceSample("):
        assert sym in syms, sym


def test_errors_without_device_are_status_codes(lib):
    """A call that needs a device returns a status (never throws / aborts)."""
    n = ctypes.c_int(-1)
    assert lib.pfdtd_device_count(ctypes.byref(n)) == 0
    if n.value == 0:
        h = ctypes.c_void_p()
        rc = lib.pfdtd_create(8, 8, 8, 0, 0, ctypes.byref(h))
        assert rc < 0 and b"device" in lib.pfdtd_last_error()
    assert lib.pfdtd_create(8, 8, 2, 0, 0, ctypes.byref(ctypes.c_void_p())) == -1
