"""Test configuration: the `gpu` marker and session-wide builds.

`-m "not gpu"` runs the oracle-vs-golden checks, the host-only API logic and
the ABI checks on any machine; `-m gpu` runs the parity tests of the CUDA
path against the oracle on a GB300.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsep.so")


@pytest.fixture(scope="session")
def lib():
    """libsep.so, built in-tree if needed."""
    from seplib_gb300 import build, load
    build.build()
    return load()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    if not lib.sep_gpu_available():
        pytest.fail("no CUDA device visible to libsep.so")
    return lib


@pytest.fixture(scope="session")
def ora():
    import oracle
    oracle.build()
    return oracle
