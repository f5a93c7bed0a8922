import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def cart():
    return ge.load_module("cartesian")


@pytest.fixture(scope="session")
def workloads():
    return ge.load_module("workloads")


@pytest.fixture(scope="session")
def orc():
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpulib(pkg):
    """The built CUDA library; GPU tests fail (not skip) if it is missing."""
    if not os.path.exists(pkg.LIB_PATH):
        pkg.build()
    return pkg.lib()
