import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def gpu_lib():
    """libpovgpu.so, built if missing; fails (no skip) when it cannot load."""
    from povray_gb300 import abi, build
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return abi.load_library()
