"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device (GB300); the
rest run on any host.  The CPU oracle is built on demand and used only as
the checker."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from melt_ibm_gb300 import abi
    return abi.Lib(oracle.build())


@pytest.fixture(scope="session")
def mibm_lib():
    """libmibm.so (built in-tree).  Fails loudly if it cannot be built."""
    from melt_ibm_gb300 import build as mbuild
    from melt_ibm_gb300 import abi
    return abi.Lib(mbuild.build())


@pytest.fixture(scope="session")
def gpu_lib(mibm_lib):
    if mibm_lib.mibm_device_count_() < 1:
        pytest.fail("marked gpu but no CUDA device is visible")
    return mibm_lib
