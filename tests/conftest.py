import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the native kernels)")


@pytest.fixture(scope="session")
def native():
    """The native library; built in-tree if missing (nvcc cross-compiles without a GPU)."""
    from gputucker_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        from gputucker_gb300 import build
        build.build()
    return _native.load()


@pytest.fixture(scope="session")
def oracle():
    import oracle_util
    return oracle_util.ora_lib()
