import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests through the C ABI")


@pytest.fixture(scope="session")
def cuda():
    """The CUDA device; GPU tests fail (never skip) without one."""
    import torch
    assert torch.cuda.is_available(), "this test needs a CUDA GPU"
    from fv3atm_gb300 import _lib
    _lib.load()
    return torch.device("cuda:0")
