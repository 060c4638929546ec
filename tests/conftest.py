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


def seed_ke(*objs, seed=3, k0=1e-4, e0=1e-5):
    """Sets the same turbulence on every object (GPU scenarios and oracles
    alike): tke and epsilon of about k0 and e0 in every cell and their depth
    integrals D Mask tke, D Mask eps, as initial forms them from the floors."""
    from nhwave_gb300 import fields as F
    rng = np.random.default_rng(seed)
    shp = objs[0].get(F.TKE).shape
    tk = k0 * (1.0 + 0.5 * rng.random(shp))
    ep = e0 * (1.0 + 0.5 * rng.random(shp))
    dm = (objs[0].get(F.D) * objs[0].get(F.MASK))[None]
    for o in objs:
        o.set(F.TKE, tk)
        o.set(F.EPS, ep)
        o.set(F.DTKE, dm * tk)
        o.set(F.DEPS, dm * ep)


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
