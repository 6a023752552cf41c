import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libmfgpu.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle.orc import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.orc import Reference
    if not Reference.available():
        pytest.skip("reference sources were not compiled here (oracle/_ref absent)")
    return Reference()


@pytest.fixture(scope="session")
def mflib():
    """The package with libmfgpu.so loaded (built in-tree if missing)."""
    from mflib_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from mflib_gb300 import build
        build.build()
    _lib.lib()
    import mflib_gb300
    return mflib_gb300


@pytest.fixture(scope="session")
def gpu(mflib):
    import ctypes
    from mflib_gb300 import _lib
    n = ctypes.c_int()
    _lib.call("mfgpu_device_count", ctypes.byref(n))
    if n.value < 1:
        pytest.skip("no CUDA device visible")
    return mflib


@pytest.fixture
def rng():
    return np.random.default_rng(20261203)
