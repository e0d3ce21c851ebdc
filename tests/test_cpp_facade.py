"""The C++ drop-in header (include/sstgraph/SparseMatrix.hpp) compiles and
links against the library (CPU), and drives the device graph (GPU)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")


def build_binary(tmp_path):
    from sstgraph_gb300 import build
    lib = build.build()
    out = os.path.join(str(tmp_path), "facade_check")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", libdir, "-lsstgraph_gb300", f"-Wl,-rpath,{libdir}", "-o", out],
                   check=True)
    return out


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_binary(tmp_path))


@pytest.mark.gpu
def test_facade_runs_on_device(tmp_path):
    out = build_binary(tmp_path)
    r = subprocess.run([out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade ok" in r.stdout
