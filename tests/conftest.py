"""pytest configuration: the `gpu` marker and the package loader.

Tests marked `gpu` need a CUDA device and run the CUDA library; the rest run
on any machine (oracle against golden vectors, host logic, library symbols).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the sm_103a library")


@pytest.fixture(scope="session")
def fk():
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx(fk):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = fk.Context(0)
    yield c
    c.close()


def rel(a, b):
    import numpy as np
    a, b = np.asarray(a), np.asarray(b)
    den = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / den
