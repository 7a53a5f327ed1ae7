"""pytest configuration: the ``gpu`` marker and shared helpers."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "vibe-model_gb300")
TESTS = os.path.dirname(os.path.abspath(__file__))
for p in (PKG, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libvibe_gb300.so")


@pytest.fixture(scope="session")
def vg():
    """The product's Python binding (raises if the CUDA library is missing)."""
    import vibe_gb300
    return vibe_gb300


@pytest.fixture(scope="session")
def oc():
    """The CPU oracle (test infrastructure)."""
    import oracle_ctypes
    if not os.path.exists(oracle_ctypes.PORT_SO):
        import subprocess
        subprocess.run(["make", "-C", oracle_ctypes.ORACLE_DIR, "-s"], check=True)
    return oracle_ctypes
