import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the product kernels")


@pytest.fixture(scope="session")
def product_lib():
    """The built libspicier_gb300.so (built here if absent; nvcc cross-compiles)."""
    from spicier_gb300 import build
    build.build()
    from spicier_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def ctx(product_lib):
    import spicier_gb300 as sg
    c = sg.Context(0)
    yield c
    c.close()
