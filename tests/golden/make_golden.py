"""Generate the committed golden fixtures from the CPU oracle.

Each fixture is a small seeded scenario advanced a few full time steps by the
oracle (the FP64 C++ restatement of the reference) with a tight Poisson
tolerance; it stores the interior of the state the parity tests compare.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from nhwave_gb300 import fields as F, scenarios as S  # noqa: E402

CASES = {"tiny_c1": 6, "tiny_c2": 6, "tiny_c3": 6, "tiny_c4": 4}
FIELDS = ("ETA", "D", "U", "V", "W", "P", "OMEGA", "MASK")
TOL = 1e-14


def make(name: str, steps: int):
    p, d, e, u = S.make(name, seed=7)
    p.tol = TOL
    p.itmax = 5000
    o = O.Oracle(p, d, e, u)
    for _ in range(steps):
        rc = o.step()
        assert rc == 0, (name, rc)
    out = {}
    for f in FIELDS:
        fid = getattr(F, f)
        out[f] = o.get(fid)[o.shape.interior(fid)]
    s = o.scalars()
    out["scalars"] = np.array([s.time, s.dt, o.mass(), s.run_step])
    return out


if __name__ == "__main__":
    for name, steps in CASES.items():
        out = make(name, steps)
        np.savez_compressed(os.path.join(HERE, f"{name}_{steps}steps.npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})
