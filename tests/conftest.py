import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (runs the product library)")
    config.addinivalue_line("markers", "slow: larger sizes")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle, build

    build()
    return Oracle()


@pytest.fixture(scope="session")
def sp():
    """The product package with its CUDA library built and loaded."""
    from spnngp_gb300.build import build

    build()
    import spnngp_gb300

    spnngp_gb300.default_context()
    return spnngp_gb300


def cm(coords):
    return np.ascontiguousarray(np.asarray(coords).T).reshape(-1)


def xorder(coords):
    return coords[np.argsort(coords[:, 0], kind="stable")]
