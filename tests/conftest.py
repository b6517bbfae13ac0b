import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the CUDA library and the oracle once per session (incremental)."""
    import __graft_entry__
    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def gpu():
    import grudon_gb300 as g
    if g.device_count() < 1:
        pytest.fail("this test needs a CUDA device; run it with -m gpu on a GPU host")
    return g
