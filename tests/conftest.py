import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the library's kernels")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session")
def built():
    """Build the library and the oracle once per session (both in-tree)."""
    from shell_gb300 import build as b
    import oracle

    b.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def cuda_ok(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return True
