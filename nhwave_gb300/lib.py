"""ctypes binding of ``libnhw_gpu.so`` -- the C-ABI of include/nhwave_gb300.h.

``Scenario`` mirrors the reference's subroutine interface for the time-step
path: one method per replaced subroutine (``estimate_dt``, ``update_mask``,
``update_vars``, ``source_terms``, ``fluxes``, ``eval_duvw(istep)``,
``sponge_damping``; src/nhwave.F:119-258), plus ``step``/``run`` for the whole
loop body and field access in the reference's ghosted Fortran layout.  There is
no CPU fallback: without the built library every call raises.
"""
from __future__ import annotations

import ctypes
import os
import warnings

import numpy as np

from . import fields as F
from .params import NhwParams, NhwScalars

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnhw_gpu.so")

OK, ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_DT_MIN, ERR_KRYLOV_NOCONV, ERR_NAN, \
    ERR_TIMEOUT, ERR_STATE, ERR_CAPACITY, ERR_NOT_FOUND = range(12)

# every entry point declared in include/nhwave_gb300.h
EXPORTS = [
    "nhw_create", "nhw_destroy", "nhw_setup", "nhw_get_field", "nhw_set_field", "nhw_field_shape",
    "nhw_get_scalars", "nhw_set_time", "nhw_set_wave_phases", "nhw_set_wave_spectrum", "nhw_estimate_dt", "nhw_update_bathymetry", "nhw_update_wave_bc",
    "nhw_update_mask",
    "nhw_update_vars", "nhw_source_terms", "nhw_fluxes", "nhw_eval_duvw", "nhw_sponge_damping",
    "nhw_eval_turb", "nhw_step", "nhw_run", "nhw_mass", "nhw_statistics", "nhw_synchronize", "nhw_run_timed", "nhw_profile",
    "nhw_profile_report", "nhw_time_smoother", "nhw_abi_sizes", "nhw_status_string", "nhw_last_error",
    "nhw_estimate_dt_noalloc",
    "nhw_ensemble_create", "nhw_ensemble_step", "nhw_ensemble_run_timed", "nhw_ensemble_tune",
    "nhw_ensemble_get_info", "nhw_ensemble_destroy", "nhw_device_bytes",
    "nhw_checkpoint_bytes", "nhw_save_state", "nhw_load_state",
]


class NhwStats(ctypes.Structure):
    """nhw_stats: the figures of the reference's statistics."""
    _fields_ = [(n, ctypes.c_double) for n in
                ("mass_volume", "energy", "max_eta", "min_eta", "max_u", "max_v", "max_w")]


class EnsembleOpts(ctypes.Structure):
    """nhw_ensemble_opts (include/nhwave_gb300.h)."""
    _fields_ = [("cells_per_block", ctypes.c_int32), ("block_rows", ctypes.c_int32),
                ("coarse_sweeps", ctypes.c_int32), ("solver", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


class EnsembleInfo(ctypes.Structure):
    """nhw_ensemble_info (include/nhwave_gb300.h)."""
    _fields_ = [("members", ctypes.c_int32), ("solve_launches_per_stage", ctypes.c_int32),
                ("blocks_per_launch", ctypes.c_int32), ("max_resident_blocks", ctypes.c_int32),
                ("kernels_per_step", ctypes.c_int64), ("cells", ctypes.c_int64), ("opts", EnsembleOpts),
                ("kernels_launched", ctypes.c_int64)]


class NhwError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = f"{where}: {status_string(status)}"
        if status == ERR_CUDA:
            msg += f" ({last_error()})"
        super().__init__(msg)


_lib = None


def load(path: str | None = None):
    """Load the library (it must have been built: ``nhwave_gb300.build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FileNotFoundError(
            f"{path} is missing: build it with nhwave_gb300.build.build() (there is no CPU fallback)")
    L = ctypes.CDLL(path)
    vp, i32, dbl = ctypes.c_void_p, ctypes.c_int32, ctypes.c_double
    P = ctypes.POINTER
    L.nhw_create.argtypes = [P(NhwParams), P(vp)]
    L.nhw_destroy.argtypes = [vp]
    L.nhw_setup.argtypes = [vp, vp, vp, vp]
    L.nhw_get_field.argtypes = [vp, i32, vp]
    L.nhw_set_field.argtypes = [vp, i32, vp]
    L.nhw_field_shape.argtypes = [vp, i32, P(i32 * 3), P(i32)]
    L.nhw_get_scalars.argtypes = [vp, P(NhwScalars)]
    L.nhw_set_time.argtypes = [vp, dbl, dbl, i32]
    L.nhw_set_wave_phases.argtypes = [vp, i32, vp]
    L.nhw_set_wave_spectrum.argtypes = [vp, i32, i32, vp, vp, vp, vp]
    for n in ("nhw_estimate_dt", "nhw_update_bathymetry", "nhw_update_wave_bc", "nhw_update_mask", "nhw_update_vars",
              "nhw_source_terms", "nhw_fluxes", "nhw_sponge_damping", "nhw_synchronize"):
        getattr(L, n).argtypes = [vp]
    L.nhw_eval_duvw.argtypes = [vp, i32]
    L.nhw_eval_turb.argtypes = [vp, i32]
    L.nhw_step.argtypes = [vp, P(dbl), P(dbl), P(i32)]
    L.nhw_run.argtypes = [vp, i32, P(i32)]
    L.nhw_mass.argtypes = [vp, P(dbl)]
    L.nhw_statistics.argtypes = [vp, P(NhwStats)]
    L.nhw_abi_sizes.argtypes = [P(i32), P(i32)]
    L.nhw_run_timed.argtypes = [vp, i32, P(dbl)]
    L.nhw_profile.argtypes = [vp, i32]
    L.nhw_profile_report.argtypes = [vp, ctypes.c_char_p, i32]
    L.nhw_time_smoother.argtypes = [vp, i32, ctypes.c_int64, P(dbl)]
    L.nhw_estimate_dt_noalloc.argtypes = [vp] * 5 + [i32] * 3 + [dbl] * 5 + [vp, vp]
    L.nhw_ensemble_create.argtypes = [P(vp), i32, P(EnsembleOpts), P(vp)]
    L.nhw_ensemble_step.argtypes = [vp, i32]
    L.nhw_ensemble_run_timed.argtypes = [vp, i32, P(dbl)]
    L.nhw_ensemble_tune.argtypes = [vp, i32, P(EnsembleOpts)]
    L.nhw_ensemble_get_info.argtypes = [vp, P(EnsembleInfo)]
    L.nhw_ensemble_destroy.argtypes = [vp]
    L.nhw_device_bytes.argtypes = [P(NhwParams), P(ctypes.c_int64)]
    L.nhw_checkpoint_bytes.argtypes = [vp, P(ctypes.c_int64)]
    L.nhw_save_state.argtypes = [vp, vp, ctypes.c_int64]
    L.nhw_load_state.argtypes = [vp, vp, ctypes.c_int64]
    L.nhw_status_string.argtypes = [ctypes.c_int]
    L.nhw_status_string.restype = ctypes.c_char_p
    L.nhw_last_error.argtypes = []
    L.nhw_last_error.restype = ctypes.c_char_p
    for n in EXPORTS:
        if n not in ("nhw_status_string", "nhw_last_error"):
            getattr(L, n).restype = ctypes.c_int
    _lib = L
    return L


def status_string(st: int) -> str:
    return load().nhw_status_string(st).decode()


def last_error() -> str:
    return load().nhw_last_error().decode()


_HARD = {ERR_ARG, ERR_UNSUPPORTED, ERR_CUDA, ERR_NOMEM, ERR_DT_MIN, ERR_NAN, ERR_TIMEOUT, ERR_STATE}


def _chk(st: int, where: str) -> int:
    if st in _HARD:
        raise NhwError(st, where)
    if st == ERR_KRYLOV_NOCONV:
        warnings.warn(f"{where}: Poisson solve stopped at ITMAX above TOL", RuntimeWarning, stacklevel=3)
    return st


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Scenario:
    """One scenario on the GPU through the C-ABI."""

    def __init__(self, params: NhwParams, depth=None, eta0=None, uvw0=None):
        L = load()
        self.params = params.copy()
        self.shape = F.Shapes(params)
        h = ctypes.c_void_p()
        _chk(L.nhw_create(ctypes.byref(self.params), ctypes.byref(h)), "nhw_create")
        self._h = h
        if depth is not None:
            self.setup(depth, eta0, uvw0)

    def setup(self, depth, eta0=None, uvw0=None):
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (depth, eta0, uvw0)]
        _chk(load().nhw_setup(self._h, *[_ptr(a) for a in keep]), "nhw_setup")

    def close(self):
        if getattr(self, "_h", None):
            load().nhw_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- the reference's subroutines
    def estimate_dt(self):
        return _chk(load().nhw_estimate_dt(self._h), "estimate_dt")

    def update_bathymetry(self):
        return _chk(load().nhw_update_bathymetry(self._h), "update_bathymetry")

    def update_wave_bc(self):
        return _chk(load().nhw_update_wave_bc(self._h), "update_wave_bc")

    def update_mask(self):
        return _chk(load().nhw_update_mask(self._h), "update_mask")

    def update_vars(self):
        return _chk(load().nhw_update_vars(self._h), "update_vars")

    def source_terms(self):
        return _chk(load().nhw_source_terms(self._h), "source_terms")

    def fluxes(self):
        return _chk(load().nhw_fluxes(self._h), "fluxes")

    def eval_duvw(self, istep: int):
        return _chk(load().nhw_eval_duvw(self._h, istep), "eval_duvw")

    def sponge_damping(self):
        return _chk(load().nhw_sponge_damping(self._h), "sponge_damping")

    def eval_turb(self, istep: int):
        return _chk(load().nhw_eval_turb(self._h, istep), "eval_turb")

    def step(self):
        return _chk(load().nhw_step(self._h, None, None, None), "nhw_step")

    def run(self, n: int) -> int:
        done = ctypes.c_int32(0)
        _chk(load().nhw_run(self._h, n, ctypes.byref(done)), "nhw_run")
        return done.value

    def save_state(self) -> np.ndarray:
        """Complete state as a byte array (nhw_save_state); resume with load_state."""
        n = ctypes.c_int64(0)
        _chk(load().nhw_checkpoint_bytes(self._h, ctypes.byref(n)), "nhw_checkpoint_bytes")
        buf = np.empty(n.value, dtype=np.uint8)
        _chk(load().nhw_save_state(self._h, buf.ctypes.data, buf.size), "nhw_save_state")
        return buf

    def load_state(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        _chk(load().nhw_load_state(self._h, buf.ctypes.data, buf.size), "nhw_load_state")

    def run_timed(self, n: int) -> float:
        """Run n steps; device milliseconds from CUDA events on the handle's stream."""
        ms = ctypes.c_double(0.0)
        _chk(load().nhw_run_timed(self._h, n, ctypes.byref(ms)), "nhw_run_timed")
        return ms.value

    def profile(self, on: bool):
        _chk(load().nhw_profile(self._h, 1 if on else 0), "nhw_profile")

    def profile_report(self) -> dict:
        """{'launches': N, 'kernels': {name: (launches, total_ms)}}"""
        L = load()
        n = L.nhw_profile_report(self._h, None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        L.nhw_profile_report(self._h, buf, n + 1)
        lines = buf.value.decode().strip().splitlines()
        out = {"launches": int(lines[0].split()[1]), "kernels": {}}
        for ln in lines[1:]:
            name, c, t = ln.split()
            out["kernels"][name] = (int(c), float(t))
        return out

    def time_smoother(self, reps: int = 50, flush_bytes: int = 256 << 20) -> float:
        """Device microseconds of one level-0 multigrid half-sweep (bulk-timed
        in a CUDA graph, the L2 evicted before each V-cycle's four)."""
        us = ctypes.c_double(0.0)
        _chk(load().nhw_time_smoother(self._h, reps, flush_bytes, ctypes.byref(us)), "nhw_time_smoother")
        return us.value

    def synchronize(self):
        return _chk(load().nhw_synchronize(self._h), "nhw_synchronize")

    def mass(self) -> float:
        m = ctypes.c_double(0.0)
        _chk(load().nhw_mass(self._h, ctypes.byref(m)), "nhw_mass")
        return m.value

    def statistics(self) -> dict:
        """nhw_statistics: MassVolume, Energy, MaxEta, MinEta, MaxU, MaxV, MaxW."""
        st = NhwStats()
        _chk(load().nhw_statistics(self._h, ctypes.byref(st)), "nhw_statistics")
        return {n: getattr(st, n) for n, _ in NhwStats._fields_}

    def scalars(self) -> NhwScalars:
        s = NhwScalars()
        _chk(load().nhw_get_scalars(self._h, ctypes.byref(s)), "nhw_get_scalars")
        return s

    def set_time(self, time: float, dt: float, run_step: int):
        _chk(load().nhw_set_time(self._h, time, dt, run_step), "nhw_set_time")

    def set_wave_spectrum(self, freq, dire, spc2d, phases=None):
        """The 2-D spectrum of LEF_SPC / INT_SPC (densities, as read_spc2d
        returns them) or INT_IRR (amplitudes and phases, as read_irr2d returns
        them) for nhw_set_wave_spectrum: spc2d and phases flat, direction fastest."""
        f, d, s = (np.ascontiguousarray(a, dtype=np.float64) for a in (freq, dire, spc2d))
        ph = None if phases is None else np.ascontiguousarray(phases, dtype=np.float64)
        _chk(load().nhw_set_wave_spectrum(self._h, f.size, d.size, _ptr(f), _ptr(d), _ptr(s), _ptr(ph)),
             "nhw_set_wave_spectrum")

    def set_wave_phases(self, phases):
        """Phases (radians) of the LEF_JON / LEF_TMA / INT_JON / INT_TMA components (nhw_set_wave_phases)."""
        a = np.ascontiguousarray(phases, dtype=np.float64)
        _chk(load().nhw_set_wave_phases(self._h, a.size, _ptr(a)), "nhw_set_wave_phases")

    def get(self, field: int, out: np.ndarray | None = None) -> np.ndarray:
        """Whole ghosted field as a [k][j][i] array (into ``out`` when given: a
        C-contiguous array of the field's size and dtype, e.g. pinned memory)."""
        shp, dtype = self.shape.of(field)
        n = int(np.prod(shp))
        if out is None:
            out = np.empty(n, dtype=dtype)
        elif out.dtype != dtype or out.size != n or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be C-contiguous {dtype} with {n} elements")
        _chk(load().nhw_get_field(self._h, field, _ptr(out)), "nhw_get_field")
        return out.reshape(shp[::-1])

    def set(self, field: int, arr):
        shp, dtype = self.shape.of(field)
        a = np.ascontiguousarray(arr, dtype=dtype).ravel()
        if a.size != int(np.prod(shp)):
            raise ValueError(f"field {F.NAMES[field]} wants {shp}, got {a.size} elements")
        _chk(load().nhw_set_field(self._h, field, _ptr(a)), "nhw_set_field")


def device_bytes(params: NhwParams) -> int:
    """Device memory a Scenario with these parameters would hold (nhw_device_bytes)."""
    b = ctypes.c_int64(0)
    _chk(load().nhw_device_bytes(ctypes.byref(params), ctypes.byref(b)), "nhw_device_bytes")
    return b.value


class Ensemble:
    """Many scenarios advanced together: one CUDA graph launch per ensemble
    step (nhw_ensemble_*).  ``members`` are set-up ``Scenario`` objects; they
    stay usable for field access, and must outlive the ensemble."""

    def __init__(self, members, cells_per_block: int = 0, block_rows: int = 0, coarse_sweeps: int = 0,
                 solver: int = 0):
        self.members = list(members)
        arr = (ctypes.c_void_p * len(self.members))(*[m._h for m in self.members])
        o = EnsembleOpts(cells_per_block, block_rows, coarse_sweeps, solver)
        self._e = ctypes.c_void_p()
        _chk(load().nhw_ensemble_create(arr, len(self.members), ctypes.byref(o), ctypes.byref(self._e)),
             "nhw_ensemble_create")

    def step(self, n: int = 1) -> int:
        return _chk(load().nhw_ensemble_step(self._e, n), "nhw_ensemble_step")

    def run_timed(self, n: int) -> float:
        ms = ctypes.c_double(0.0)
        _chk(load().nhw_ensemble_run_timed(self._e, n, ctypes.byref(ms)), "nhw_ensemble_run_timed")
        return ms.value

    def tune(self, steps_per_trial: int = 1) -> EnsembleOpts:
        o = EnsembleOpts()
        _chk(load().nhw_ensemble_tune(self._e, steps_per_trial, ctypes.byref(o)), "nhw_ensemble_tune")
        return o

    def info(self) -> EnsembleInfo:
        out = EnsembleInfo()
        _chk(load().nhw_ensemble_get_info(self._e, ctypes.byref(out)), "nhw_ensemble_get_info")
        return out

    def close(self):
        if getattr(self, "_e", None) and self._e.value:
            load().nhw_ensemble_destroy(self._e)
            self._e = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
