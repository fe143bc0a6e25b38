"""The C-ABI library loads and exports every entry point its headers declare
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "ucm-mpi-gpu_gb300", "gpb", "libgpb.so")


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gpb\w*|computeGPb|getCudaDeviceCount|gpbSetTextonCodebook)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from gpb import build
        build.build()
    return ctypes.CDLL(LIB)


def test_c_symbols_exported(lib):
    names = _declared("gpb.h")
    assert "gpb_compute_batch" in names and "gpb_create" in names
    for n in names:
        assert hasattr(lib, n), n


def test_damascene_signatures_exported():
    # computeGPb / getCudaDeviceCount keep their C++ signatures
    # (damascene/include/globalPb.h:35,44), so they are exported mangled
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True).stdout
    assert "_Z10computeGPbjjjPjPPfS1_" in out
    assert "_Z18getCudaDeviceCountv" in out
    assert "_Z20gpbSetTextonCodebookPKfi" in out
    for n in _declared("gpb_damascene.h"):
        assert n in out


def test_status_strings(lib):
    lib.gpb_status_str.restype = ctypes.c_char_p
    assert lib.gpb_status_str(0) == b"ok"
    assert lib.gpb_status_str(4) == b"eigensolver did not converge"


def test_default_params(lib):
    import gpb
    p = gpb.default_params()
    assert p.nvec == 9 and p.krylov_dim > p.krylov_keep >= p.nvec
    assert p.compat == gpb.COMPAT_CPU and p.eig_mode == gpb.EIG_LANCZOS
    assert 0 < p.eig_tol <= 1e-4
