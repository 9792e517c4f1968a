"""The C++ facade (include/pinocchio_gb300.hpp) with the reference's
rneaInParallel / abaInParallel argument shapes: it compiles against the C ABI
(CPU) and round-trips ABA(RNEA(a)) = a with host column-major matrices and the
reference's pool-size check (GPU)."""
import os
import subprocess

import pytest

from pinocchio_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "facade_check.cpp")


def build_exe(tmp_path):
    _build.build()
    exe = str(tmp_path / "facade_check")
    libdir = os.path.dirname(_build.LIB)
    cuda = os.path.dirname(os.path.dirname(_build.nvcc()))
    cmd = ["g++", "-std=c++17", "-O1", "-o", exe, SRC, f"-I{cuda}/include", f"-L{libdir}", "-lpinocchio_gb300",
           f"-Wl,-rpath,{libdir}", f"-L{cuda}/lib64", "-lcudart", f"-Wl,-rpath,{cuda}/lib64"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_exe(tmp_path))


@pytest.mark.gpu
def test_facade_roundtrip_on_gpu(tmp_path):
    r = subprocess.run([build_exe(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "pool_check_ok" in r.stdout
    assert "single_calls" in r.stdout and "size_check_ok" in r.stdout
