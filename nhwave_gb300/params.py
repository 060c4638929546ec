"""Run-time parameters of the time-step path, mirroring ``nhw_params`` in
``include/nhwave_gb300.h`` field for field.

The keys are the ``input.txt`` keys that the reference reads in
``read_input`` (src/initialize.F:141-1321); :func:`read_input` parses the same
``KEY = value`` format (src/mod_util.F:8-463: the first ``=`` splits key and
value, ``!`` starts a comment, a missing required key is an error, floats are
read as double).
"""
from __future__ import annotations

import ctypes

NHW_FP64 = 0
NHW_FP32_IR = 1
(WM_NONE, WM_INT_LIN, WM_INT_SOL, WM_LEF_LIN, WM_LEF_SOL, WM_LEF_STK, WM_LEF_CON, WM_WAV_CUR, WM_FOCUSED,
 WM_LEF_TID, WM_RIG_LIN, WM_FLUX_LR, WM_LEF_JON, WM_LEF_TMA, WM_LEF_SPC, WM_INT_CON, WM_INT_JON, WM_INT_TMA,
 WM_INT_SPC, WM_INT_IRR) = range(20)
# fed through the west boundary (BC_X0 = 3)
WM_LEF = (WM_LEF_LIN, WM_LEF_SOL, WM_LEF_STK, WM_LEF_CON, WM_WAV_CUR, WM_FOCUSED, WM_LEF_TID, WM_FLUX_LR,
          WM_LEF_JON, WM_LEF_TMA, WM_LEF_SPC)
# fed through the east boundary (BC_Xn = 3)
WM_EAST = (WM_RIG_LIN, WM_FLUX_LR)
# internal source strips (src/source_terms.F)
WM_INT = (WM_INT_LIN, WM_INT_SOL, WM_INT_CON, WM_INT_JON, WM_INT_TMA, WM_INT_SPC, WM_INT_IRR)
WM_OTHER = -1   # a wavemaker of the reference outside this path (rejected by nhw_create)
SLIDE_NONE, SLIDE_RIGID_3D = 0, 1
DEPTH_CELL_CENTER, DEPTH_CELL_GRID = 0, 1


class NhwParams(ctypes.Structure):
    """ctypes image of ``nhw_params`` (natural alignment, as the C compiler lays it out)."""

    _fields_ = [
        ("Mglob", ctypes.c_int32), ("Nglob", ctypes.c_int32), ("Kglob", ctypes.c_int32),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double),
        ("ivgrd", ctypes.c_int32), ("grd_r", ctypes.c_double),
        ("dt_ini", ctypes.c_double), ("dt_min", ctypes.c_double), ("dt_max", ctypes.c_double),
        ("total_time", ctypes.c_double), ("sim_steps", ctypes.c_int32),
        ("cfl", ctypes.c_double),
        ("froude_cap_on", ctypes.c_int32), ("froude_cap", ctypes.c_double),
        ("min_dep", ctypes.c_double),
        ("non_hydro", ctypes.c_int32), ("time_order", ctypes.c_int32),
        ("hllc", ctypes.c_int32), ("viscous_flow", ctypes.c_int32), ("barotropic", ctypes.c_int32),
        ("itmax", ctypes.c_int32), ("tol", ctypes.c_double),
        ("bc_x0", ctypes.c_int32), ("bc_xn", ctypes.c_int32), ("bc_y0", ctypes.c_int32),
        ("bc_yn", ctypes.c_int32), ("bc_z0", ctypes.c_int32),
        ("visc", ctypes.c_double), ("slat", ctypes.c_double),
        ("wind_u", ctypes.c_double), ("wind_v", ctypes.c_double),
        ("depth_type", ctypes.c_int32), ("wavemaker", ctypes.c_int32),
        ("amp_wave", ctypes.c_double), ("per_wave", ctypes.c_double), ("dep_wave", ctypes.c_double),
        ("theta_wave", ctypes.c_double), ("cur_wave", ctypes.c_double),
        ("xsource_west", ctypes.c_double), ("xsource_east", ctypes.c_double),
        ("ysource_suth", ctypes.c_double), ("ysource_nrth", ctypes.c_double),
        ("sponge_on", ctypes.c_int32),
        ("sponge_west_width", ctypes.c_double), ("sponge_east_width", ctypes.c_double),
        ("sponge_south_width", ctypes.c_double), ("sponge_north_width", ctypes.c_double),
        ("tramp", ctypes.c_double),
        ("slide_type", ctypes.c_int32),
        ("slide_t", ctypes.c_double), ("slide_l", ctypes.c_double), ("slide_w", ctypes.c_double),
        ("slide_angle", ctypes.c_double), ("slope_angle", ctypes.c_double),
        ("slide_x0", ctypes.c_double), ("slide_y0", ctypes.c_double),
        ("slide_ut", ctypes.c_double), ("slide_a0", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("precond", ctypes.c_int32),
        ("mg_weight", ctypes.c_float),
        ("krylov_kernel", ctypes.c_int32),
        ("mg_coarse_sweeps", ctypes.c_int32),
        ("mg_cta_columns", ctypes.c_int32),
        ("mg_aggregate", ctypes.c_int32),
        ("test_barrier_extra", ctypes.c_int32),
        ("ivturb", ctypes.c_int32), ("ihturb", ctypes.c_int32), ("rng", ctypes.c_int32),
        ("cvs", ctypes.c_double), ("chs", ctypes.c_double), ("schmidt", ctypes.c_double),
        ("viscous_number", ctypes.c_double),
        ("ibot", ctypes.c_int32), ("cd0", ctypes.c_double), ("zob", ctypes.c_double),
        ("nwave", ctypes.c_int32), ("component_amp_type", ctypes.c_int32),
        ("k_center", ctypes.c_double), ("f_center", ctypes.c_double), ("x_breaking", ctypes.c_double),
        ("t_breaking", ctypes.c_double), ("slope_group", ctypes.c_double),
        ("normalized_delta_f", ctypes.c_double), ("depth_comp", ctypes.c_double),
        ("sd_return", ctypes.c_double),
        ("hm0", ctypes.c_double), ("tp", ctypes.c_double), ("freq_min", ctypes.c_double),
        ("freq_max", ctypes.c_double), ("numfreq", ctypes.c_int32), ("wave_seed", ctypes.c_int32),
        ("prod_type", ctypes.c_int32),
    ]

    def copy(self) -> "NhwParams":
        out = NhwParams()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(self))
        return out

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class NhwScalars(ctypes.Structure):
    """ctypes image of ``nhw_scalars``."""

    _fields_ = [
        ("time", ctypes.c_double), ("dt", ctypes.c_double), ("dt_old", ctypes.c_double),
        ("run_step", ctypes.c_int32), ("last_krylov_iters", ctypes.c_int32),
        ("total_krylov_iters", ctypes.c_int64), ("poisson_solves", ctypes.c_int64),
        ("last_rel_residual", ctypes.c_double), ("last_refinements", ctypes.c_int32),
        ("status", ctypes.c_int32),
    ]


def default_params(**kw) -> NhwParams:
    """Defaults of the reference's own input.txt for the keys on the path, then ``kw``."""
    p = NhwParams()
    p.Mglob, p.Nglob, p.Kglob = 64, 4, 5
    p.dx = p.dy = 1.0
    p.ivgrd, p.grd_r = 1, 1.1
    p.dt_ini, p.dt_min, p.dt_max = 0.01, 1e-5, 60.0
    p.total_time, p.sim_steps = 1.0e30, 2**31 - 1
    p.cfl = 0.5
    p.froude_cap_on, p.froude_cap = 1, 100.0
    p.min_dep = 0.01
    p.non_hydro, p.time_order, p.hllc, p.viscous_flow, p.barotropic = 1, 3, 0, 0, 1
    p.itmax, p.tol = 1000, 1e-8
    p.bc_x0 = p.bc_xn = p.bc_y0 = p.bc_yn = p.bc_z0 = 1
    p.visc, p.slat, p.wind_u, p.wind_v = 1e-6, 0.0, 0.0, 0.0
    p.depth_type, p.wavemaker = DEPTH_CELL_CENTER, WM_NONE
    p.sponge_on = 0
    p.slide_type = SLIDE_NONE
    p.precision = NHW_FP64
    p.ivturb = p.ihturb = 1
    p.prod_type = 3
    p.cvs = p.chs = 0.0
    p.schmidt, p.viscous_number = 1.0, 1.0 / 6.0
    p.ibot, p.cd0, p.zob = 1, 0.0, 1e-4
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(f"unknown nhw_params field {k!r}")
        setattr(p, k, v)
    return p


# --------------------------------------------------------------- input.txt
_REQUIRED = ("Mglob", "Nglob", "Kglob", "DX", "DY", "DT_INI", "DT_MIN", "DT_MAX", "CFL", "MinDep")


def _parse_kv(path: str) -> dict:
    vals = {}
    with open(path, "r", errors="replace") as fh:
        for line in fh:
            line = line.split("!", 1)[0]
            if "=" not in line:
                continue
            key, val = line.split("=", 1)
            key, val = key.strip(), val.strip()
            if key and key not in vals:  # the first occurrence wins, as Extract_Val_String
                vals[key] = val
    return vals


def _logical(v: str) -> int:
    return 1 if v.strip().upper().lstrip(".").startswith("T") else 0


def read_input(path: str) -> NhwParams:
    """Parse an NHWAVE ``input.txt`` into :class:`NhwParams` (keys on this path only)."""
    kv = _parse_kv(path)
    for k in _REQUIRED:
        if k not in kv:
            raise ValueError(f"error reading variable: {k} does not exist in file: {path}")

    def f(k, d=None):
        return float(kv[k]) if k in kv else d

    def i(k, d=None):
        return int(float(kv[k])) if k in kv else d

    def s(k, d=""):
        return kv.get(k, d).strip().strip("'\"")

    p = default_params()
    p.Mglob, p.Nglob, p.Kglob = i("Mglob"), i("Nglob"), i("Kglob")
    p.dx, p.dy = f("DX"), f("DY")
    p.ivgrd, p.grd_r = i("IVGRD", 1), f("GRD_R", 1.1)
    p.dt_ini, p.dt_min, p.dt_max = f("DT_INI"), f("DT_MIN"), f("DT_MAX")
    p.total_time = f("TOTAL_TIME", 1e30)
    p.sim_steps = i("SIM_STEPS", 2**31 - 1)
    p.cfl, p.min_dep = f("CFL"), f("MinDep")
    p.froude_cap = f("FROUDE_CAP", 100.0)
    p.non_hydro = _logical(kv.get("NON_HYDRO", "F"))
    to = s("TIME_ORDER", "THIRD").upper()
    p.time_order = 3 if to.startswith("THI") else 2 if to.startswith("SEC") else 1
    p.hllc = _logical(kv.get("HLLC", "F"))
    p.viscous_flow = _logical(kv.get("VISCOUS_FLOW", "F"))
    p.barotropic = _logical(kv.get("BAROTROPIC", "T"))
    p.itmax, p.tol = i("ITMAX", 1000), f("TOL", 1e-8)
    p.bc_x0, p.bc_xn = i("BC_X0", 1), i("BC_Xn", 1)
    p.bc_y0, p.bc_yn = i("BC_Y0", 1), i("BC_Yn", 1)
    p.bc_z0 = i("BC_Z0", 1)
    p.ibot, p.cd0, p.zob = i("Ibot", 1), f("Cd0", 0.0), f("Zob", 1e-4)
    p.visc, p.slat = f("VISCOSITY", 1e-6), f("slat", 0.0)
    if p.viscous_flow:
        p.ivturb, p.ihturb, p.rng = i("IVTURB", 1), i("IHTURB", 1), _logical(kv.get("RNG", "F"))
        p.cvs, p.chs, p.schmidt = f("Cvs", 0.0), f("Chs", 0.0), f("Schmidt", 1.0)
        p.viscous_number = f("VISCOUS_NUMBER", 1.0 / 6.0)
        p.prod_type = i("PRODTYPE", 3)
    p.wind_u, p.wind_v = f("WindU", 0.0), f("WindV", 0.0)
    dt_ = s("DEPTH_TYPE", "CELL_CENTER").upper()
    p.depth_type = DEPTH_CELL_GRID if dt_ == "CELL_GRID" else DEPTH_CELL_CENTER
    wm = s("WAVEMAKER", "NONE").upper()
    # a generator of the reference that this path does not build is kept as
    # WM_OTHER and rejected, not run as NONE
    known = {"NONE": WM_NONE, "INT_LIN": WM_INT_LIN, "INT_SOL": WM_INT_SOL, "LEF_LIN": WM_LEF_LIN,
             "LEF_SOL": WM_LEF_SOL, "LEF_STK": WM_LEF_STK, "LEF_CON": WM_LEF_CON, "WAV_CUR": WM_WAV_CUR,
             "FOCUSED": WM_FOCUSED, "LEF_TID": WM_LEF_TID, "RIG_LIN": WM_RIG_LIN, "FLUX_LR": WM_FLUX_LR,
             "LEF_JON": WM_LEF_JON, "LEF_TMA": WM_LEF_TMA, "LEF_SPC": WM_LEF_SPC, "INT_CON": WM_INT_CON,
             "INT_JON": WM_INT_JON, "INT_TMA": WM_INT_TMA, "INT_SPC": WM_INT_SPC, "INT_IRR": WM_INT_IRR}
    p.wavemaker = known.get(wm[:7], WM_OTHER) if wm else WM_NONE
    if wm[:3] in ("LEF", "RIG", "INT", "FLU", "WAV"):
        p.amp_wave, p.per_wave, p.dep_wave = f("AMP", 0.0), f("PER", 1.0), f("DEP", 1.0)
        p.theta_wave, p.cur_wave = f("THETA", 0.0), f("CUR", 0.0)
        p.sd_return = f("sd_return", 0.0)
        if wm[:3] == "INT":
            p.xsource_west, p.xsource_east = f("Xsource_West", 0.0), f("Xsource_East", 0.0)
            p.ysource_suth, p.ysource_nrth = f("Ysource_Suth", 0.0), f("Ysource_Nrth", 0.0)
    if wm[4:7] in ("JON", "TMA"):   # WaveMaker(5:7), src/initialize.F:888-892
        p.hm0, p.tp = f("Hm0", 0.0), f("Tp", 0.0)
        p.freq_min, p.freq_max, p.numfreq = f("Freq_Min", 0.0), f("Freq_Max", 0.0), i("NumFreq", 0)
    if wm[:3] == "FOC":   # src/initialize.F:709-719
        p.nwave, p.component_amp_type = i("nwave", 0), i("Component_Amp_Type", 1)
        p.k_center, p.f_center = f("k_center", 0.0), f("f_center", 0.0)
        p.x_breaking, p.t_breaking = f("x_breaking", 0.0), f("t_breaking", 0.0)
        p.slope_group, p.normalized_delta_f = f("Slope_group", 0.0), f("normalized_delta_f", 0.0)
        p.depth_comp = f("depth_comp", 0.0)
    p.sponge_on = _logical(kv.get("SPONGE_ON", "F"))
    if p.sponge_on:
        p.sponge_west_width = f("Sponge_West_Width", 0.0)
        p.sponge_east_width = f("Sponge_East_Width", 0.0)
        p.sponge_south_width = f("Sponge_South_Width", 0.0)
        p.sponge_north_width = f("Sponge_North_Width", 0.0)
    p.tramp = f("TRAMP", 0.0)
    # The reference reads SlideType only in a build with its landslide option
    # (src/initialize.F:1033-1045), and its example inputs carry the key as a
    # template line (TWOLAYER in the submerged bar, berkhoff and breaking
    # cases, which have no slide).  RIGID_3D, the slide this path builds,
    # turns the slide on; any other value reads as no slide, as in a build
    # without that option.
    st = s("SlideType", "").upper()
    if st.startswith("RIGID_3D"):
        p.slide_type = SLIDE_RIGID_3D
        p.slide_t, p.slide_l, p.slide_w = f("SlideT"), f("SlideL"), f("SlideW")
        p.slide_angle, p.slope_angle = f("SlideAngle", 0.0), f("SlopeAngle", 0.0)
        p.slide_x0, p.slide_y0 = f("SlideX0"), f("SlideY0")
        p.slide_ut, p.slide_a0 = f("SlideUt"), f("SlideA0")
    return p


def read_spc2d(path: str):
    """The 2-D spectrum file of LEF_SPC (src/initialize.F:783-819): NumFreq
    and NumDir, then NumFreq frequencies, NumDir directions and the
    NumFreq x NumDir densities, direction fastest.  Returns (freq, dire,
    spc2d) as float64 arrays, spc2d flat in that order (as nhw_set_wave_spectrum
    takes it)."""
    import numpy as np
    with open(path) as fh:
        vals = fh.read().split()
    nf, nd = int(float(vals[0])), int(float(vals[1]))
    rest = np.array([float(v) for v in vals[2:2 + nf + nd + nf * nd]])
    if rest.size != nf + nd + nf * nd:
        raise ValueError(f"{path}: expected {nf} + {nd} + {nf * nd} values after the counts")
    return rest[:nf].copy(), rest[nf:nf + nd].copy(), rest[nf + nd:].copy()


def read_irr2d(path: str):
    """The component file of INT_IRR (src/initialize.F:835-876): NumFreq and
    NumDir, then NumFreq frequencies, NumDir directions, the NumFreq x NumDir
    component amplitudes and as many phases, direction fastest.  Returns
    (freq, dire, amp, phases) as float64 arrays, amp and phases flat in that
    order (as nhw_set_wave_spectrum takes them)."""
    import numpy as np
    with open(path) as fh:
        vals = fh.read().split()
    nf, nd = int(float(vals[0])), int(float(vals[1]))
    n = nf + nd + 2 * nf * nd
    rest = np.array([float(v) for v in vals[2:2 + n]])
    if rest.size != n:
        raise ValueError(f"{path}: expected {nf} + {nd} + 2 x {nf * nd} values after the counts")
    a = nf + nd
    return rest[:nf].copy(), rest[nf:a].copy(), rest[a:a + nf * nd].copy(), rest[a + nf * nd:].copy()


def unsupported_reason(p: NhwParams) -> str | None:
    """Why a parameter set falls outside this path (None when it is inside)."""
    if p.viscous_flow and (p.ivturb not in (1, 2, 3, 10, 20, 30) or not (p.ihturb in (1, 2) or p.ihturb >= 10)):
        return (f"VISCOUS_FLOW=T with IVTURB={p.ivturb}, IHTURB={p.ihturb} (the GPU path has IVTURB 1 constant, 2 "
                "subgrid, 3 and 10 k-epsilon, 20 and 30 LES, and IHTURB 1, 2 or >= 10)")
    if p.wavemaker not in (WM_NONE,) + WM_INT + WM_LEF + WM_EAST:
        return ("WAVEMAKER (only NONE, INT_LIN, INT_SOL, INT_CON, INT_JON, INT_TMA, INT_SPC, INT_IRR, LEF_LIN, "
                "LEF_SOL, LEF_STK, LEF_CON, LEF_TID, LEF_JON, LEF_TMA, LEF_SPC, WAV_CUR, FOCUSED, RIG_LIN and "
                "FLUX_LR are on the GPU path)")
    if p.bc_x0 == 3 and p.wavemaker not in WM_LEF:
        return ("BC_X0=3 needs a LEF_LIN, LEF_SOL, LEF_STK, LEF_CON, LEF_TID, LEF_JON, LEF_TMA, LEF_SPC, WAV_CUR, "
                "FOCUSED or FLUX_LR wavemaker")
    if p.bc_xn == 3 and p.wavemaker not in WM_EAST:
        return "BC_Xn=3 needs the RIG_LIN or FLUX_LR wavemaker"
    for name in ("bc_x0", "bc_xn", "bc_y0", "bc_yn"):
        ok = {"bc_x0": (1, 2, 3, 5), "bc_xn": (1, 2, 3, 5, 6)}.get(name, (1, 2, 5))
        if getattr(p, name) not in ok:
            return (f"{name.upper()}={getattr(p, name)} (walls 1/2, wall friction 5, the inflows 3 "
                    "and the east Orlanski boundary 6 are on the GPU path)")
    if p.wavemaker == WM_FLUX_LR and not p.zob > 0:
        return "FLUX_LR needs Zob > 0 (its inflow has a logarithmic profile)"
    if p.bc_z0 not in (1, 2, 5):
        return f"BC_Z0={p.bc_z0} (free slip 1, no slip 2 and the friction law 5 are on the GPU path)"
    if 5 in (p.bc_z0, p.bc_x0, p.bc_xn, p.bc_y0, p.bc_yn) and p.ibot not in (1, 2):
        return f"Ibot={p.ibot} (1 drag coefficient, 2 roughness height)"
    return None


def cells(p: NhwParams) -> int:
    return int(p.Mglob) * int(p.Nglob) * int(p.Kglob)


__all__ = [
    "NhwParams", "NhwScalars", "default_params", "read_input", "unsupported_reason", "cells",
    "NHW_FP64", "NHW_FP32_IR", "WM_NONE", "WM_INT_LIN", "WM_INT_SOL", "WM_LEF_LIN", "WM_LEF_SOL",
    "WM_LEF_STK", "WM_LEF_CON", "WM_WAV_CUR", "WM_FOCUSED", "WM_LEF_TID", "WM_LEF",
    "WM_RIG_LIN", "WM_FLUX_LR", "WM_LEF_JON", "WM_LEF_TMA", "WM_LEF_SPC", "WM_EAST", "read_spc2d",
    "WM_INT_CON", "WM_INT_JON", "WM_INT_TMA", "WM_INT_SPC", "WM_INT_IRR", "WM_INT", "read_irr2d",
    "WM_OTHER",
    "SLIDE_NONE",
    "SLIDE_RIGID_3D", "DEPTH_CELL_CENTER", "DEPTH_CELL_GRID",
]
