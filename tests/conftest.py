import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built CUDA library")


@pytest.fixture(scope="session")
def built():
    """Build the native libraries (and the oracle port) once per session."""
    from cbns3d_cart_mpi_gb300 import build as b
    from oracle.build import build_port
    b.build()
    build_port()
    return True


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN
