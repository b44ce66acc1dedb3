import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libdftg.so")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    if not _has_gpu():
        pytest.skip("no CUDA device")
    from dftcxx_gb300 import build, _lib
    build.build()
    return _lib.load()
