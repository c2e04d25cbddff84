import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libpmx.so')


@pytest.fixture(scope='session', autouse=True)
def libpmx():
    """libpmx.so, built in-tree when missing (nvcc cross-compiles without a
    GPU): the host-side growth integrator lives in it too."""
    from pmwd_gb300 import _build, _lib
    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.load()


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail('CUDA is required for gpu-marked tests')
    from pmwd_gb300 import _lib
    _lib.load()
    return torch.device('cuda', 0)
