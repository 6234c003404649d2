import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libfdsgpu.so")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def gpu():
    """The CUDA device; builds libfdsgpu.so if needed. Skips only when no GPU is
    visible; a missing or broken library fails the test."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pyfds_gb300 import _build, _capi
    _build.build()
    _capi.load()
    return torch.device("cuda", 0)
