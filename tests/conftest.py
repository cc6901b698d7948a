import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle (and, where its sources exist, the pinned reference)
    and the engine library once per session."""
    import oracle
    oracle.build(ref=True)
    from fft3dcl_gb300 import build
    build.build()
    yield
