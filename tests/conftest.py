"""Test configuration: import paths, the `gpu` marker and shared fixtures."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
PKG_DIR = REPO / "speo-gpu-single-control_gb300"
for p in (str(PKG_DIR), str(REPO / "oracle"), str(REPO)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import speo_oracle

    speo_oracle.lib()
    return speo_oracle


@pytest.fixture(scope="session")
def lib():
    from speo_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def _device_error_flags_clean(request):
    """After every GPU test: the library's device error flags must be clear (read and reset)."""
    yield
    if request.node.get_closest_marker("gpu") is None:
        return
    import ctypes

    import torch

    if not torch.cuda.is_available():
        return
    from speo_gb300 import _lib

    bits = ctypes.c_uint32(0)
    st = _lib.load().speo_device_error_bits(ctypes.byref(bits))
    assert st == 0, f"speo_device_error_bits failed: {st}"
    assert bits.value == 0, f"device error flags 0x{bits.value:x} set by {request.node.nodeid}"
