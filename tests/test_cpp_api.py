"""The C++ host API (include/panopaea.hpp): it compiles against the C ABI
header and links against the library on the CPU; on the GPU the compiled
test (tests/cpp/test_api.cpp -- the reference's own grid.rs tests, the PCG
and the step loop of its example, and the error behaviour) runs and
passes."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from panopaea_gb300 import build as B

    lib = B.build()
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    exe = str(tmp_path / "test_api")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "tests", "golden"), os.path.join(ROOT, "tests", "cpp", "test_api.cpp"),
           "-L" + os.path.dirname(lib), "-lpanopaea_gpu", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    assert "warning" not in p.stderr, p.stderr
    return exe


def test_cpp_api_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_cpp_api_reference_tests_pass(tmp_path):
    exe = _build(tmp_path)
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0 and "ALL OK" in p.stdout, p.stdout + p.stderr
