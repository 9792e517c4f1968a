"""The integer FP32 <-> FP64 conversions the mixed kernels use instead of the
hardware conversions (csrc/gb_spatial.cuh widen / narrow): a CUDA test program
compares them with the hardware casts over edge cases and 200k seeded bit
patterns (it compiles here; it runs on a GPU)."""
import os
import shutil
import subprocess

import pytest

from pinocchio_gb300 import _build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cuda", "conversions_check.cu")


def build_exe(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "conversions_check")
    subprocess.run([nvcc, *_build.ARCH, "-O2", "-std=c++17", "-o", exe, SRC], check=True, capture_output=True, text=True)
    return exe


def test_conversion_check_compiles(tmp_path):
    assert os.path.exists(build_exe(tmp_path))


@pytest.mark.gpu
def test_conversions_match_hardware(tmp_path):
    r = subprocess.run([build_exe(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "conversions_ok" in r.stdout
