import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def solrt():
    build = importlib.import_module("sol-rs_gb300.build")
    build.build_lib()
    return importlib.import_module("sol-rs_gb300")


@pytest.fixture(scope="session")
def oracle(solrt):
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def ctx(solrt):
    c = solrt.Context(0)
    yield c
    c.close()
