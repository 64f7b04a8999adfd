"""Shared fixtures: the package (liblbmgpu.so via ctypes) and the FP64 oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as ge

    b = ge._import_build_module()
    b.build()
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle


GOLDEN = os.path.join(ROOT, "tests", "golden")
