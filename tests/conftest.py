import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def gpu_lib():
    """The built library on a machine with a GPU; fails (does not skip) otherwise."""
    from pansim_gb300 import native
    L = native.lib()
    assert native.device_count() > 0, "no CUDA device visible"
    return L
