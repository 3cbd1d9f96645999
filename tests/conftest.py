"""Test configuration: the ``gpu`` marker and shared fixtures.

``-m "not gpu"`` runs on any host (oracle vs golden vectors, host logic, the
C-ABI library loads and exports its symbols).  ``-m gpu`` needs a CUDA device
and runs the parity tests through the C ABI.
"""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a CUDA device is required for -m gpu tests")
    return torch


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
