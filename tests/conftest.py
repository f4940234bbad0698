import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def package():
    """The product package (its directory name is not an identifier)."""
    return importlib.import_module("assemble-them-all_gb300")


def submodule(name):
    return importlib.import_module(f"assemble-them-all_gb300.{name}")


@pytest.fixture(scope="session")
def workloads():
    return submodule("workloads")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O
