import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs through libzeta_cuda.so)")
    config.addinivalue_line("markers", "slow: larger parity sweeps")


@pytest.fixture(scope="session")
def zeta_device():
    """Initialise libzeta_cuda.so on cuda:0 once per session (GPU tests only)."""
    import zeta_gb300 as z
    z.init(0, 64, 16)
    yield z
    z.release()
