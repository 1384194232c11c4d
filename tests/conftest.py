import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgclaw.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import ref

    ref.lib()
    return ref


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a GPU")
    from clawpack_gb300 import _lib

    _lib.lib()
    _lib.lib(strict=True)
    return torch.device("cuda:0")
