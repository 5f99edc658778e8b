import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built CUDA library")


def _cuda_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def orc():
    """The CPU oracle (C restatement of the 1x1 LU path)."""
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def sl():
    """The GPU library's Python mirror; the CUDA library must be built."""
    import scalapack_gb300 as S

    S.lib()
    return S


@pytest.fixture(scope="session")
def gpu_required():
    if not _cuda_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return True
