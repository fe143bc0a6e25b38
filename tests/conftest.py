import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "ucm-mpi-gpu_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def orc():
    import pyoracle
    if not os.path.exists(pyoracle.LIBORC):
        import subprocess
        subprocess.run(["make", "-s", "-f", "oracle/Makefile"], cwd=ROOT, check=True)
    return pyoracle


@pytest.fixture(scope="session")
def ref(orc):
    if not orc.ref_available():
        pytest.skip("reference cores (oracle/_ref) not built on this machine")
    return orc
