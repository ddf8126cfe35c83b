import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a GB300 (CUDA device) and the built library")


@pytest.fixture(scope="session")
def gb():
    """The CUDA library (built in-tree); fails loudly if it is missing."""
    import ludwig_gb300
    if not os.path.exists(ludwig_gb300.LIB_PATH):
        ludwig_gb300.build()
    ludwig_gb300.load_library()
    return ludwig_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    oracle.lib()
    return oracle
