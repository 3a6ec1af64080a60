"""Shared fixtures. Tests marked `gpu` need a CUDA device and libhalapt.so;
everything else runs on the CPU (oracle, host logic, ABI surface)."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libhalapt.so")


@pytest.fixture(scope="session")
def pt():
    """The product package (directory name has a hyphen, so import by name)."""
    return importlib.import_module("hala-pathtracer_gb300")


@pytest.fixture(scope="session")
def abi(pt):
    return importlib.import_module("hala-pathtracer_gb300.abi")


@pytest.fixture(scope="session")
def scenes(pt):
    return importlib.import_module("hala-pathtracer_gb300.scenes")


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_lib(pt):
    """Builds (if needed) and loads libhalapt.so; fails loudly when it cannot."""
    pt.build()
    return pt.load_library()
