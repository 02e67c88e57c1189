import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libplk (nvcc cross-compiles without a GPU) and the oracle."""
    from phylommand_gb300 import build
    from oracle import oracle
    build.build()
    oracle.load()
    yield
