import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def aniso_mesh():
    d = np.load(os.path.join(GOLDEN, "cube_anisotropic_mesh.npz"))
    return d["ndglno"].astype(np.int32), d["coords"].astype(np.float64)


@pytest.fixture(scope="session")
def goldens():
    return dict(np.load(os.path.join(GOLDEN, "oracle_goldens.npz")))


def row_scaled_error(a, b, findrm):
    """max_i max_j |a_ij - b_ij| / max_j |b_ij| over rows (row-scaled relative error)."""
    a = np.asarray(a)
    b = np.asarray(b)
    n = findrm.size - 1
    rows = np.repeat(np.arange(n), np.diff(findrm))
    rowmax = np.zeros(n)
    np.maximum.at(rowmax, rows, np.abs(b))
    rowmax[rowmax == 0] = 1.0
    return float(np.max(np.abs(a - b) / rowmax[rows])) if a.size else 0.0
