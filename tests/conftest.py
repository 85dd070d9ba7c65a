import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on the device)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def lib():
    from lightne_gb300 import _lib
    from lightne_gb300 import build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def ctx(lib):
    from lightne_gb300.api import Context
    c = Context(0)
    yield c
    c.close()
