import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def qmin():
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def oracle():
    import qmin_oracle
    qmin_oracle.build()
    return qmin_oracle
