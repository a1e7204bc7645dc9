"""Shared pytest setup: the `gpu` marker, import paths and fixtures."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def msq():
    """The product's Python host layer (loads libmsq_cuda.so)."""
    return importlib.import_module("mixed-mlx_gb300")


@pytest.fixture(scope="session")
def ctx(msq):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = msq.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden_codecs():
    return np.load(os.path.join(GOLDEN, "codecs.npz"))


@pytest.fixture(scope="session")
def golden_numerics():
    return np.load(os.path.join(GOLDEN, "numerics.npz"))
