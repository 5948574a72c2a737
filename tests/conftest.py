import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


def cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not cuda_available():
        pytest.fail("this test needs a CUDA GPU")
    import ptwalker_gb300 as ptw
    ptw.load_library()
    return ptw


@pytest.fixture(scope="session")
def s16_edges():
    import oracle
    return oracle.rmat_clean_edges(16, 16, 0.57, 0.19, 0.19, 1)


@pytest.fixture(scope="session")
def s16_canon(s16_edges):
    import oracle
    return oracle.canonical_from_edges(*s16_edges)
