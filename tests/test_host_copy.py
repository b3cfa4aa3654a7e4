"""The host copy pool (libqdt_gb300/csrc/host_copy.cu) on the CPU: single
large copies split over the pool, gathers of many small arrays, and several
threads copying at once, compared byte for byte. The harness
(host_copy_check.cpp) is compiled with g++ against the library's source."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "libqdt_gb300", "csrc")


def test_parallel_copy_exact(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "host_copy_check")
    cmd = [gxx, "-O2", "-std=c++17", "-I", CSRC, "-x", "c++", os.path.join(HERE, "host_copy_check.cpp"),
           "-x", "c++", os.path.join(CSRC, "host_copy.cu"), "-o", exe, "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0 concurrent bad 0" in r.stdout
