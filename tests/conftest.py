import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in-tree if it is missing (nvcc cross-compiles)."""
    from pmmc_gb300 import build, capi
    if not os.path.exists(capi.LIB_PATH):
        build.build()
    return capi.lib()


@pytest.fixture(scope="session")
def ctx(built_lib):
    from pmmc_gb300 import capi
    c = capi.Context(0)
    yield c
    c.close()
