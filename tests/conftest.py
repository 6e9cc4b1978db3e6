import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(REPO, "lidar-processing-v2_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Shared objects are built by __graft_entry__.build(); build here when missing or stale."""
    sys.path.insert(0, REPO)
    import __graft_entry__

    __graft_entry__.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import lidar_gb300 as lp

    c = lp.Context(0)
    yield c
    c.close()
