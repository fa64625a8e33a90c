"""Shared pytest configuration: the ``gpu`` marker and common fixtures."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libsmileigb300.so")


@pytest.fixture(scope="session")
def golden_ops():
    z = np.load(os.path.join(GOLDEN, "operators.npz"))
    cases = {}
    for key in z.files:
        case, name = key.split("/", 1)
        cases.setdefault(case, {})[name] = z[key]
    return cases


@pytest.fixture(scope="session")
def golden_rad():
    z = np.load(os.path.join(GOLDEN, "radiation.npz"))
    return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def cpu_oracle():
    import oracle
    return oracle.Oracle()


def rel_err(a, b):
    """max|a - b| / max|b| -- the parity metric (J has near-zero nodes)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = float(np.max(np.abs(b))) if b.size else 0.0
    return float(np.max(np.abs(a - b))) / (m if m > 0 else 1.0) if b.size else 0.0
