"""Test configuration: the `gpu` marker, the repo on sys.path, and library builds.

`-m "not gpu"` tests run anywhere (oracle against the reference's golden vectors, host logic,
the C-ABI library's exports); `-m gpu` tests need a CUDA device and compare the engine with the
oracle."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def engine_lib():
    """The engine's C-ABI library, built in-tree if missing."""
    from micrographia_gb300 import _abi, build

    build.build()
    return _abi.lib()


@pytest.fixture(scope="session")
def O():
    """The oracle module (compiled on first use)."""
    from oracle import oracle

    oracle.lib()
    return oracle
