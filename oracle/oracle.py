"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE.

The oracle (``oracle/nhw_oracle.cpp``) is a plain FP64 C++ restatement of the
reference's time-step routines, used as the checker in ``tests/``, in
``__graft_entry__.smoke()`` and as the CPU baseline in ``bench.py``.  Nothing in
the product package imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, REPO)

from nhwave_gb300.params import NhwParams, NhwScalars  # noqa: E402
from nhwave_gb300 import fields as F  # noqa: E402

SRC = os.path.join(HERE, "nhw_oracle.cpp")
LIB = os.path.join(HERE, "_build", "liboracle.so")
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    """Compile the oracle into ``oracle/_build/liboracle.so`` (g++, no build system)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    hdr = os.path.join(REPO, "include", "nhwave_gb300.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-o", tmp, SRC])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        vp, i32, dbl = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(NhwParams), ctypes.POINTER(i32)]
        L.orc_destroy.argtypes = [vp]
        L.orc_setup.argtypes = [vp, vp, vp, vp]
        for name in ("orc_estimate_dt", "orc_step"):
            getattr(L, name).argtypes = [vp]
        L.orc_eval_duvw.argtypes = [vp, i32]
        L.orc_eval_turb.argtypes = [vp, i32]
        L.orc_eval_turb.restype = None
        for name in ("orc_update_bathymetry", "orc_update_wave_bc", "orc_update_mask", "orc_update_vars",
                     "orc_source_terms", "orc_fluxes", "orc_sponge_damping",
                     "orc_generate_coef_rhs"):
            getattr(L, name).argtypes = [vp]
            getattr(L, name).restype = None
        L.orc_mass.argtypes = [vp]
        L.orc_mass.restype = dbl
        L.orc_statistics.argtypes = [vp, ctypes.c_void_p]
        L.orc_statistics.restype = None
        L.orc_get_field.argtypes = [vp, i32, vp]
        L.orc_set_field.argtypes = [vp, i32, vp]
        L.orc_get_scalars.argtypes = [vp, ctypes.POINTER(NhwScalars)]
        L.orc_get_scalars.restype = None
        L.orc_set_time.argtypes = [vp, dbl, dbl, i32]
        L.orc_set_time.restype = None
        L.orc_get_grid.argtypes = [vp, i32, vp]
        L.orc_get_coef.argtypes = [vp, vp, vp]
        L.orc_limiter.argtypes = [dbl, dbl]
        L.orc_limiter.restype = dbl
        L.orc_wave_number.argtypes = [vp, dbl]
        L.orc_wave_number.restype = dbl
        L.orc_elliptic.argtypes = [i32, dbl, dbl]
        L.orc_elliptic.restype = dbl
        L.orc_set_wave_phases.argtypes = [vp, i32, vp]
        L.orc_set_wave_spectrum.argtypes = [vp, i32, i32, vp, vp, vp, vp]
        L.orc_get_inflow_eta.argtypes = [vp, vp]
        L.orc_cnoidal_wave.argtypes = [dbl, dbl, dbl, vp]
        L.orc_cnoidal_wave.restype = i32
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


STAT_KEYS = ("mass_volume", "energy", "max_eta", "min_eta", "max_u", "max_v", "max_w")


class Oracle:
    """One scenario on the CPU oracle; method names follow the reference subroutines."""

    def __init__(self, params: NhwParams, depth, eta0=None, uvw0=None):
        L = lib()
        self.params = params.copy()
        st = ctypes.c_int(0)
        self._h = L.orc_create(ctypes.byref(self.params), ctypes.byref(st))
        if not self._h:
            raise ValueError(f"oracle rejected parameters (status {st.value})")
        self._keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                      for a in (depth, eta0, uvw0)]
        rc = L.orc_setup(self._h, *[_ptr(a) for a in self._keep])
        if rc:
            raise RuntimeError(f"orc_setup failed: {rc}")
        self.shape = F.Shapes(params)

    def close(self):
        if self._h:
            lib().orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # reference subroutines
    def estimate_dt(self):
        return lib().orc_estimate_dt(self._h)

    def update_bathymetry(self):
        lib().orc_update_bathymetry(self._h)

    def update_wave_bc(self):
        lib().orc_update_wave_bc(self._h)

    def update_mask(self):
        lib().orc_update_mask(self._h)

    def update_vars(self):
        lib().orc_update_vars(self._h)

    def source_terms(self):
        lib().orc_source_terms(self._h)

    def fluxes(self):
        lib().orc_fluxes(self._h)

    def eval_duvw(self, istep: int):
        return lib().orc_eval_duvw(self._h, istep)

    def sponge_damping(self):
        lib().orc_sponge_damping(self._h)

    def eval_turb(self, istep: int):
        lib().orc_eval_turb(self._h, istep)

    def step(self):
        return lib().orc_step(self._h)

    def run(self, n: int):
        for _ in range(n):
            rc = self.step()
            if rc not in (0, 6):
                return rc
        return 0

    def mass(self) -> float:
        return lib().orc_mass(self._h)

    def statistics(self) -> dict:
        """statistics' figures (src/nhwave.F:3118-3160), in the reference's loop order."""
        out = np.zeros(7)
        lib().orc_statistics(self._h, out.ctypes.data)
        return dict(zip(STAT_KEYS, out.tolist()))

    def scalars(self) -> NhwScalars:
        s = NhwScalars()
        lib().orc_get_scalars(self._h, ctypes.byref(s))
        return s

    def set_time(self, time, dt, run_step):
        lib().orc_set_time(self._h, time, dt, run_step)

    def set_wave_phases(self, phases):
        a = np.ascontiguousarray(phases, dtype=np.float64)
        rc = lib().orc_set_wave_phases(self._h, a.size, _ptr(a))
        if rc:
            raise ValueError("set_wave_phases: not a LEF_JON / LEF_TMA scenario of that many components")

    def set_wave_spectrum(self, freq, dire, spc2d, phases=None):
        f, d, s = (np.ascontiguousarray(a, dtype=np.float64) for a in (freq, dire, spc2d))
        self._spc = (f, d, s, None if phases is None else np.ascontiguousarray(phases, dtype=np.float64))
        rc = lib().orc_set_wave_spectrum(self._h, f.size, d.size, _ptr(f), _ptr(d), _ptr(s), _ptr(self._spc[3]))
        if rc:
            raise ValueError("set_wave_spectrum: not a LEF_SPC / INT_SPC / INT_IRR scenario, fewer than 2 "
                             "frequencies / directions, an internal maker's direction beyond 90 degrees, or "
                             "INT_IRR without phases")

    def inflow_eta(self) -> np.ndarray:
        """Ein_X0 of the last update_wave_bc (all Nloc rows)."""
        out = np.empty(self.shape.Nloc)
        lib().orc_get_inflow_eta(self._h, _ptr(out))
        return out

    def get(self, field: int) -> np.ndarray:
        shp, dtype = self.shape.of(field)
        out = np.empty(int(np.prod(shp)), dtype=dtype)
        rc = lib().orc_get_field(self._h, field, _ptr(out))
        if rc:
            raise ValueError(f"bad field {field}")
        return out.reshape(shp[::-1])  # [k][j][i] view of the Fortran array

    def set(self, field: int, arr: np.ndarray):
        shp, dtype = self.shape.of(field)
        a = np.ascontiguousarray(arr, dtype=dtype).ravel()
        assert a.size == int(np.prod(shp))
        lib().orc_set_field(self._h, field, _ptr(a))

    def grid(self, which: int) -> np.ndarray:
        n = {0: self.shape.Mloc + 1, 1: self.shape.Mloc, 2: self.shape.Nloc + 1,
             3: self.shape.Nloc, 4: self.shape.Kloc + 1, 5: self.shape.Kloc, 6: self.shape.Kloc}[which]
        out = np.empty(n)
        lib().orc_get_grid(self._h, which, _ptr(out))
        return out

    def coef_rhs(self):
        n = int(self.params.Mglob * self.params.Nglob * self.params.Kglob)
        coef = np.empty(15 * n)
        rhs = np.empty(n)
        lib().orc_get_coef(self._h, _ptr(coef), _ptr(rhs))
        return coef.reshape(15, n), rhs


def limiter(a: float, b: float) -> float:
    return lib().orc_limiter(a, b)


BATHY_FIELDS = ("HC", "HFX", "HFY", "HFX0", "HFY0", "DELXH", "DELYH", "DELTH", "DELT2H")


def run_scenario(name: str, steps: int, tol: float = 1e-13, pinned: bool = False, seed: int = 7,
                 fields=("ETA", "D", "U", "V", "W", "P", "MASK"), **kw) -> dict:
    """Run the seeded scenario ``name`` (``nhwave_gb300.scenarios.make``) for
    ``steps`` FP64 steps and return plain arrays, so that a process pool can
    run it beside the GPU: the end ``fields`` (whole ghosted arrays), the
    mask after every step, the scalars, and -- with ``pinned`` -- each step's
    bathymetry right after update_bathymetry (the step is then taken routine
    by routine in the main loop's order, src/nhwave.F:127-258), for a GPU run
    that copies it in."""
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make(name, seed=seed, **kw)
    p.tol, p.itmax, p.precision = tol, 20000, 0
    o = Oracle(p, d, e, u)
    masks, bathy = [], []
    for _ in range(steps):
        if pinned:
            rc = o.estimate_dt()
            if rc:
                raise RuntimeError(f"oracle estimate_dt: {rc}")
            o.update_bathymetry()
            bathy.append({n: o.get(getattr(F, n)).copy() for n in BATHY_FIELDS})
            o.update_mask()
            o.update_vars()
            for s in (1, 2, 3):
                o.source_terms()
                o.fluxes()
                rc = o.eval_duvw(s)
                if rc:
                    raise RuntimeError(f"oracle eval_duvw: {rc}")
                if o.params.sponge_on:
                    o.sponge_damping()
                o.eval_turb(s)
        else:
            rc = o.step()
            if rc:
                raise RuntimeError(f"oracle step: {rc}")
        masks.append(o.get(F.MASK).copy())
    sc = o.scalars()
    out = {"fields": {f: o.get(getattr(F, f)).copy() for f in fields}, "masks": masks, "bathy": bathy,
           "time": sc.time, "dt": sc.dt, "run_step": sc.run_step}
    o.close()
    return out
