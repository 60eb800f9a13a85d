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


_CUDART = []


def _cudart():
    """The CUDA runtime the library links (the toolkit's libcudart), or None."""
    if not _CUDART:
        import ctypes
        import glob
        lib = None
        for pat in ("/usr/local/cuda/lib64/libcudart.so*",
                    "/usr/local/cuda/targets/*/lib/libcudart.so*"):
            for f in sorted(glob.glob(pat)):
                try:
                    lib = ctypes.CDLL(f)
                    break
                except OSError:
                    continue
            if lib is not None:
                break
        _CUDART.append(lib)
    return _CUDART[0]


@pytest.fixture(autouse=True)
def no_pending_cuda_error(request):
    """After each GPU test, no CUDA runtime error is left pending on the test's thread: a call
    the library made and failed without reading back would otherwise surface in a later,
    unrelated call."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    rt = _cudart()
    if rt is None:
        return
    code = rt.cudaGetLastError()
    assert code == 0, "CUDA error %d left pending" % code
