import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a GB300 (runs the CUDA path through the C-ABI)")
    config.addinivalue_line(
        "markers", "slow: a longer CPU-side check")


def load_case(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def quadrature(K):
    """The reference's own tables (tests/golden/quadratures.npz)."""
    key = {1: ("1_gl", "2_1_gl"), 2: ("2_gl", "4_2_gl"), 3: ("2_gl", "4_3_gl"),
           5: ("3_gl", "6_5_gl"), 6: ("3_gl", "6_6_gl")}[K]
    with np.load(os.path.join(GOLDEN, "quadratures.npz")) as z:
        return z["weights_" + key[1]], z["samples_" + key[0]]


@pytest.fixture
def case():
    return load_case
