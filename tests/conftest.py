import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs through libmulskips_gpu.so)")
    config.addinivalue_line("markers", "slow: long CPU oracle runs")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import ora
    ora.build()
    return ora


@pytest.fixture(scope="session")
def engine_lib():
    """The CUDA engine library; must already be built (no fallback)."""
    from mulskips_gb300 import _native
    return _native.lib()
