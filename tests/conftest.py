"""Shared helpers of the test suite.

Markers: ``gpu`` -- needs a CUDA device (the parity tests proper; they call the
C-ABI library).  Everything else runs on the CPU: the oracle against known
answers and the committed golden fixtures, host logic, and that the C-ABI
library loads and exports every declared symbol.
"""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C-ABI)")


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0.0:
        return num
    return num / den


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    from nhwave_gb300 import build, lib
    build.build()
    return lib.load()
