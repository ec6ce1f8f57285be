import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbba.so")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gb():
    return importlib.import_module("3dreconstruction_gb300")


@pytest.fixture(scope="session")
def abi():
    return importlib.import_module("3dreconstruction_gb300.abi")


@pytest.fixture(scope="session")
def scenes():
    return importlib.import_module("3dreconstruction_gb300.scenes")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def handle(gb):
    if not gpu_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    h = gb.Handle(0)
    yield h
    h.close()


def load_golden(name):
    import numpy as np
    path = os.path.join(GOLDEN, name)
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}
