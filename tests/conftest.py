import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "open-3d-wallturbulence_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")


@pytest.fixture(scope="session")
def port_lib():
    """The CPU oracle restatement, built on demand (g++, a few seconds)."""
    from oracle import PORT_LIB
    subprocess.run(["make", "-s", "-C", ORACLE, "port"], check=True)
    return PORT_LIB


@pytest.fixture(scope="session")
def gpu_lib():
    """libowt_gpu.so, built on demand (nvcc)."""
    from owt.build import build
    return build()


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
