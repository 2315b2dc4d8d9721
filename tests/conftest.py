import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "methodoflines.jl_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmolgpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library on a GPU machine; GPU tests fail loudly if it is missing."""
    from molgpu import _lib as L
    lib = L.lib()
    return lib
