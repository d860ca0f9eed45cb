import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pd-ipc-armadillodemo_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and the built CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    """Builds libpdipc.so if it is missing or stale and returns its path."""
    from pdipc import build
    return build.build()
