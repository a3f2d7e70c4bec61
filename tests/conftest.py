import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; the gpu tests go through it."""
    from alamo_gb300 import build
    build.build()
    from alamo_gb300 import _lib
    return _lib.lib()
