import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "parallel-fast-marching-method_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfm3dt_gpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built if needed; GPU tests fail loudly without it."""
    from fm3dt import build as fb
    fb.build()
    import fm3dt
    return fm3dt.load()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle
