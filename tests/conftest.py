"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
SMALL_CASES = ["regular2_q4", "cube2_q1", "cube2_q2", "cube2_q3", "cube3_q4", "cube2_q6", "cube2_q8", "cube4_q4"]
# the same kind of runs with the order-4 modified-equation leap-frog
ORDER4_CASES = ["cube2_q2_o4", "cube3_q4_o4", "cube2_q8_o4"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(params=SMALL_CASES)
def golden_case(request):
    return request.param, load_golden(request.param)


@pytest.fixture(params=ORDER4_CASES)
def golden_case4(request):
    return request.param, load_golden(request.param)


def rel_l2(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
