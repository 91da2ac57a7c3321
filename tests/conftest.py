import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; GPU tests fail loudly if it is missing."""
    from bamf_gb300 import abi, build
    build.build()
    L = abi.lib()
    assert L.bamf_device_count() > 0, "no CUDA device visible"
    return L


@pytest.fixture(scope="session")
def oracle_port():
    import oracle
    oracle.build(ref=False)
    return oracle
