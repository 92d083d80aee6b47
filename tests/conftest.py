import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the product library and the oracle once if they are missing."""
    from ether_gb300 import abi, build
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    from oracle import pyoracle
    if not os.path.exists(pyoracle.SO):
        pyoracle.build()
