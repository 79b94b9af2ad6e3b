"""Test configuration: the `gpu` marker and shared fixtures.

GPU tests call the CUDA library through its C ABI and compare with the CPU
oracle; CPU tests cover the oracle against the reference's known answers,
the host-side logic, and the library's exported symbols.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build
    build.build()
    return oracle


@pytest.fixture(scope="session")
def native():
    """The CUDA library, built if needed; GPU tests fail loudly when it cannot load."""
    from fractalpathtracer_gb300 import build, native as nat
    build.build()
    nat.lib()
    return nat
