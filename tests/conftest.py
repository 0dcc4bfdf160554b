import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "heom-quick2_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle and the product's CUDA library (no-op when current)."""
    import build_lib
    import oracle_ffi

    oracle_ffi.build()
    build_lib.build()
    yield
