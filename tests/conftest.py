import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib():
    from mdsm_gb300 import build
    build.build()
    import mdsm_gb300
    return mdsm_gb300.load()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build(reference=os.path.isdir(oracle.REF_TREE))
    return oracle


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch
