import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and the built library")


@pytest.fixture(scope="session")
def gpu_ctx():
    """One idb context for the GPU tests (fails loudly if the library is missing)."""
    from immunodbscan_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
