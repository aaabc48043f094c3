import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def skinny_lib():
    """The built libskinny.so (compiled on first use)."""
    from skinny_matmul_gb300 import build, lib
    build.build()
    return lib.load()


@pytest.fixture(scope="session")
def handle():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from skinny_matmul_gb300 import build
    build.build()
    from skinny_matmul_gb300 import Handle
    h = Handle(0)
    yield h
    h.close()
