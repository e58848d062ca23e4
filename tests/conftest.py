import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libbna.so and the oracle library if they are missing or stale."""
    from cuda_newest20160331_gb300 import build as b
    import oracle.build as ob
    b.build()
    ob.build()


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def builder():
    if not _have_gpu():
        pytest.skip("no CUDA device")
    import cuda_newest20160331_gb300 as bna
    b = bna.Builder(0)
    yield b
    b.close()
