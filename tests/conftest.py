"""Shared fixtures: the package (directory ``da-gtm_gb300``), the CPU oracle
(the checker) and the golden vectors decoded from the reference's sample
output."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "oil_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def load_pkg():
    return importlib.import_module("da-gtm_gb300")


@pytest.fixture(scope="session")
def pkg():
    return load_pkg()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def built_lib():
    """Build the CUDA library (cross-compiles without a GPU)."""
    b = importlib.import_module("da-gtm_gb300.build")
    return b.build()
