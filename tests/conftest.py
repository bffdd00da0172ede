import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; runs the sm_103a kernels through the C ABI")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build(ref=None)
    return oracle


@pytest.fixture(scope="session")
def built_lib():
    from dawgs_gb300 import build
    build.build()
    from dawgs_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def cuda(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
