import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def ghlib():
    """The built C ABI library (built in-tree on first use)."""
    import gpuheap_gb300 as gh
    if not os.path.exists(gh.library_path):
        gh.build()
    return gh.lib()
