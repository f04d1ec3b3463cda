import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def femtc():
    """The femtc_gb300 package with its library built and loaded."""
    import femtc_gb300
    femtc_gb300.load()
    return femtc_gb300


@pytest.fixture(scope="session")
def dev():
    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle
