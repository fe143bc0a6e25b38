"""The host-side dense linear algebra of the eigensolvers
(csrc/eig_host.cpp), built by the host compiler with the library's flags."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_host_dense_eigensolver(tmp_path):
    """csrc/eig_host.cpp: the symmetric eigensolver, the 32 x 32 product
    helper and the Loewdin orthonormalisation of the block solver, built with
    the library's host flags (-O3, no FMA contraction)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "eig_host_check")
    subprocess.run([cxx, "-O3", "-ffp-contract=off", "-std=c++17",
                    os.path.join(ROOT, "tests", "eig_host_check.cpp"),
                    os.path.join(ROOT, "ucm-mpi-gpu_gb300", "csrc", "eig_host.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and "ok" in out.stdout, out.stdout + out.stderr
