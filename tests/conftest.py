import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_built():
    from oracle.build import build_oracle
    build_oracle()
    return True


@pytest.fixture(scope="session")
def cuda_lib():
    from lbffs_gb300 import build as b
    b.build()
    import lbffs_gb300
    return lbffs_gb300.load_library()
