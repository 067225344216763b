import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def gbla_lib():
    """The built libgbla.so (built here if missing, never replaced by a fallback)."""
    from gputils_gb300 import build, _lib

    build.build_lib()
    return _lib.lib()


@pytest.fixture(scope="session")
def cuda(gbla_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test started without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
