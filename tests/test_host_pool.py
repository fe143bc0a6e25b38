"""The host thread pool (csrc/host_pool.h), built on its own with the host
compiler: every item runs once, an item's exception reaches the caller
after the other items are done, and the pool stays usable."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_pool(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "host_pool_check")
    subprocess.run([cxx, "-O1", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "ucm-mpi-gpu_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "host_pool_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
