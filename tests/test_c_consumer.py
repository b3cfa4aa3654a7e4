"""A C program written against include/qdt.h alone (tests/c_consumer)
compiles with a C compiler, links against the GB300 library as a client of
the reference library would, and passes its interface checks: the checks
that make no batch call here, all of them on the GPU."""
import os
import shutil
import subprocess

import pytest

import libqdt_gb300 as G
from libqdt_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c_consumer", "qdt_consumer.c")


def compile_consumer(out_dir):
    lib = G.load()   # builds the library if needed
    del lib
    cc = shutil.which("cc") or shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    exe = os.path.join(out_dir, "qdt_consumer")
    cmd = [cc, "-std=c99", "-O1", "-Wall", "-Werror", "-I", B.INCLUDE, SRC, "-o", exe, "-L", B.BUILD,
           "-lqdt_gb300", "-Wl,-rpath," + B.BUILD, "-lpthread", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_consumer_compiles_links_and_runs_host_checks(tmp_path):
    exe = compile_consumer(str(tmp_path))
    r = subprocess.run([exe, "--no-gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


@pytest.mark.gpu
def test_consumer_all_checks_on_gpu(tmp_path):
    exe = compile_consumer(str(tmp_path))
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout
