"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and libgsa.so built for it."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgsa.so")


@pytest.fixture(scope="session")
def gsa():
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a test marked gpu ran without a CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def _device_status_after_gpu_tests(request):
    """After every gpu test: no bounded device-side wait gave up (gsa_check_device_status)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import torch
    if not torch.cuda.is_available():
        return
    import __graft_entry__
    gsa = __graft_entry__.load_package()
    lib = gsa._lib.load()
    import ctypes
    st = lib.gsa_check_device_status(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, f"device status {st}: {gsa._lib.last_error()}"
