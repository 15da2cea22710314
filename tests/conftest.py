import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_api():
    """The CPU oracle library bound with the C-ABI call surface (test checker)."""
    from oracle import build as ob
    from rift_gb300 import capi
    lib = ctypes.CDLL(ob.build_oracle())
    return lib, capi.bind(lib, "rift_oracle_", create_has_mode=True)


@pytest.fixture(scope="session")
def engine_api():
    from rift_gb300 import build as eb
    from rift_gb300 import capi
    eb.build()
    return capi.load_product()
