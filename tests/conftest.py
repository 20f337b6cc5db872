import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


def pytest_collection_modifyitems(config, items):
    # GPU tests need the CUDA library; they are selected with -m gpu.
    pass


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    return oracle
