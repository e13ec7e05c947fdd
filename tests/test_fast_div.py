"""The invariant-divisor magic numbers of the index splits (fast_div in
pg_internal.cuh), checked on the CPU: a host-only program built with nvcc
compares the quotient the kernels compute against integer division for
every divisor up to 70000, powers of two and their neighbours, and 20000
random divisors, at edge and random indices over the whole 32-bit range."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fast_div_exact(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fast_div_check")
    src = os.path.join(ROOT, "tests", "cpp", "fast_div_check.cu")
    inc = ["-I" + os.path.join(ROOT, "panopaea_gb300", "csrc"), "-I" + os.path.join(ROOT, "include")]
    p = subprocess.run([nvcc, "-std=c++17", "-O2", *inc, src, "-o", exe], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and " 0 wrong" in r.stdout, r.stdout + r.stderr
