import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the sm_103a build")


@pytest.fixture(scope="session", autouse=True)
def _native_build():
    """Compile the native libraries once per session (incremental)."""
    from gpu_index_test_gb300 import build

    build.build()
    yield
