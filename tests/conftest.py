import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def built():
    """Builds the CUDA library, its host-side check library and the C oracle (once per session)."""
    from dfpsr_gb300 import build as b
    from oracle import port
    b.build()
    b.build_hostcheck()
    port.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import dfpsr_gb300 as d
    c = d.Context(0)
    yield c
    c.close()
