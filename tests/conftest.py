import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device; runs the hot path through the C ABI")


@pytest.fixture(scope="session")
def gbl():
    """The lattice library, built in tree (nvcc cross-compiles without a GPU)."""
    from banjo_gb300 import build, lattice

    build.build()
    return lattice


@pytest.fixture(scope="session")
def port():
    import oracle

    oracle.build_port()
    return oracle


@pytest.fixture(scope="session")
def device(gbl):
    if not gbl.available():
        pytest.fail("GPU test needs a CUDA device: " + gbl.description())
    return gbl
