"""The autotuner's bookkeeping (csrc/autotune.h), built by the host compiler
against a stand-in for the CUDA event calls it makes."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_autotuner_bookkeeping(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "autotune_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-I", os.path.join(ROOT, "tests", "fake_cuda"),
                    "-I", os.path.join(ROOT, "ucm-mpi-gpu_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "autotune_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "ok" in out.stdout, out.stdout + out.stderr

