import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built libmmsp_gpu.so")
    config.addinivalue_line("markers", "slow: full-size configuration")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pf_oracle

    pf_oracle.lib()
    return pf_oracle


@pytest.fixture(scope="session")
def gpu():
    """The native library on a CUDA device; fails (never skips) when absent."""
    from mmsp_gb300 import native

    L = native.load()
    return native
