import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def _gpu_available() -> bool:
    try:
        import ctypes
        ctypes.CDLL("libcuda.so.1")
    except OSError:
        return False
    return True


@pytest.fixture(scope="session")
def native():
    """The C-ABI library (built on demand). Fails loudly when it cannot load."""
    from visacd_gb300 import build, _native
    build.build_gpu()
    return _native


@pytest.fixture(scope="session")
def ctx(native):
    c = native.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def orc():
    import oracle
    return oracle
