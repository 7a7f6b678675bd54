import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels through the C ABI")
    config.addinivalue_line("markers", "slow: long-running")


def have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def m2():
    """The engine binding; builds the library if needed (fails loudly if it cannot)."""
    import mersenne2gpu_gb300 as pkg
    from mersenne2gpu_gb300 import build as b
    b.build()
    return pkg


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
