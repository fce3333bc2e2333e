"""Shared fixtures.  `-m gpu` tests need a CUDA GPU and build the native library in-tree first;
everything else runs on the CPU (oracle, golden vectors, host logic, library loading)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle32():
    from oracle import oracle
    oracle.build(with_ref=None)
    return oracle.Oracle("f32")


@pytest.fixture(scope="session")
def oracle64():
    from oracle import oracle
    oracle.build(with_ref=None)
    return oracle.Oracle("f64")


@pytest.fixture(scope="session")
def native_lib():
    from optixsoltracedemos_gb300 import build
    build.build()
    from optixsoltracedemos_gb300 import native
    return native.load()


@pytest.fixture(scope="session")
def gpu(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return native_lib
