"""CPU: the reference's own MATLAB gateway (matlab/mex_FDTD.cpp) compiles
against this library's drop-in headers (include/pfdtd/), links with
libpfdtd.so and runs its argument check, under a stand-in MEX API
(tests/mex_stub/).  Skipped where the reference tree is absent."""
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "mex_stub"))
import build_gateway  # noqa: E402


def _lib_built():
    from parallelfdtd_gb300 import build as B
    return os.path.exists(os.path.join(os.path.dirname(B.__file__), "libpfdtd.so"))


def _gateway_present():
    ref = build_gateway.reference_dir()
    return ref is not None and os.path.exists(build_gateway.gateway_source(ref))


@pytest.mark.skipif(not _gateway_present(), reason="reference tree not present")
def test_reference_mex_gateway_compiles_links_and_runs(tmp_path):
    if not _lib_built():
        pytest.skip("libpfdtd.so not built")
    exe = build_gateway.build(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2, r.stdout + r.stderr
    assert "Parse input arguments" in r.stdout
    assert "Not enough input argumets" in r.stdout  # the gateway's own message


def test_log_msg_formats(tmp_path):
    """log_msg<level>(L"...") % args, the reference's C++ logging call
    (src/logger.h:46-84), with boost::format's directives."""
    if not _lib_built():
        pytest.skip("libpfdtd.so not built")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "log.cpp"
    src.write_text(r'''
#include "logger.h"
#include <string>
int main() {
  setLogLevel(LOG_INFO);
  log_msg<LOG_INFO>(L"steps %1%, dx %2%, name %3%") % 3u % 0.125f % std::string("room");
  log_msg<LOG_WARNING>(L"%d nodes, %.3f s, %s, 100%%") % -42 % 1.23456 % "x";
  log_msg<LOG_DEBUG>(L"hidden %1%") % 1;
  return 0;
}
''')
    lib = os.path.join(repo, "parallelfdtd_gb300")
    exe = tmp_path / "log"
    subprocess.run(["g++", "-std=c++11", "-I" + os.path.join(repo, "include", "pfdtd"), str(src),
                    "-L" + lib, "-lpfdtd", "-Wl,-rpath," + lib, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    assert r.stderr.splitlines() == ["[pfdtd INFO] steps 3, dx 0.125, name room",
                                     "[pfdtd WARNING] -42 nodes, 1.235 s, x, 100%"]
