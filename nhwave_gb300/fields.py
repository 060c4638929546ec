"""Field ids of ``enum nhw_field`` (include/nhwave_gb300.h) and their shapes.

Shapes are the reference's ghosted allocations (src/initialize.F:1423-1643):
cell arrays (Mloc, Nloc[, Kloc]), x-face arrays (Mloc1, Nloc[, Kloc]), y-face
arrays (Mloc, Nloc1[, Kloc]) and z-face arrays (Mloc, Nloc, Kloc1), Fortran
order (i fastest).
"""
from __future__ import annotations

import numpy as np

NAMES = [
    "D", "D0", "ETA", "ETA0", "HC", "HC0", "DELXH", "DELYH", "DELXETA", "DELYETA", "DELTH",
    "DELT2H", "SOURCEX", "SOURCEY", "SOURCEC", "SPONGE", "R1",
    "HFX", "HFX0", "ETAXL", "ETAXR",
    "HFY", "HFY0", "ETAYL", "ETAYR",
    "MASK", "MASK_STRUCT", "MASK9",
    "U", "V", "W", "DU", "DV", "DW", "DU0", "DV0", "DW0", "P",
    "OMEGA",
    "EX", "FX", "GX", "HX",
    "EY", "FY", "GY", "HY",
    "FZ", "GZ", "HZ",
    "CMUVT", "CMUHT",
    "TKE", "EPS", "DTKE", "DEPS",
]
for _i, _n in enumerate(NAMES):
    globals()[_n] = _i
COUNT = len(NAMES)

# shape classes
C2, X2, Y2, I2, C3, Z3, X3, Y3 = range(8)
_CLASS = {}
for _n in ("D", "D0", "ETA", "ETA0", "HC", "HC0", "DELXH", "DELYH", "DELXETA", "DELYETA",
           "DELTH", "DELT2H", "SOURCEX", "SOURCEY", "SOURCEC", "SPONGE", "R1"):
    _CLASS[_n] = C2
for _n in ("HFX", "HFX0", "ETAXL", "ETAXR"):
    _CLASS[_n] = X2
for _n in ("HFY", "HFY0", "ETAYL", "ETAYR"):
    _CLASS[_n] = Y2
for _n in ("MASK", "MASK_STRUCT", "MASK9"):
    _CLASS[_n] = I2
for _n in ("U", "V", "W", "DU", "DV", "DW", "DU0", "DV0", "DW0", "P", "CMUVT", "CMUHT", "TKE", "EPS", "DTKE",
           "DEPS"):
    _CLASS[_n] = C3
for _n in ("OMEGA", "FZ", "GZ", "HZ"):
    _CLASS[_n] = Z3
for _n in ("EX", "FX", "GX", "HX"):
    _CLASS[_n] = X3
for _n in ("EY", "FY", "GY", "HY"):
    _CLASS[_n] = Y3
CLASS = [_CLASS[n] for n in NAMES]
NG = 2


class Shapes:
    """Ghosted extents of one scenario."""

    def __init__(self, p):
        self.M, self.N, self.K = int(p.Mglob), int(p.Nglob), int(p.Kglob)
        self.Mloc, self.Nloc, self.Kloc = self.M + 2 * NG, self.N + 2 * NG, self.K + 2 * NG

    def of(self, field: int):
        c = CLASS[field]
        Ml, Nl, Kl = self.Mloc, self.Nloc, self.Kloc
        shp = {C2: (Ml, Nl), X2: (Ml + 1, Nl), Y2: (Ml, Nl + 1), I2: (Ml, Nl),
               C3: (Ml, Nl, Kl), Z3: (Ml, Nl, Kl + 1), X3: (Ml + 1, Nl, Kl),
               Y3: (Ml, Nl + 1, Kl)}[c]
        return shp, (np.int32 if c == I2 else np.float64)

    def interior(self, field: int):
        """Index tuple selecting the interior of a [k][j][i] view (faces: all interior faces)."""
        c = CLASS[field]
        i0, j0, k0 = NG, NG, NG
        si = slice(i0, i0 + self.M + (1 if c in (X2, X3) else 0))
        sj = slice(j0, j0 + self.N + (1 if c in (Y2, Y3) else 0))
        sk = slice(k0, k0 + self.K + (1 if c == Z3 else 0))
        if c in (C2, X2, Y2, I2):
            return (sj, si)
        return (sk, sj, si)
