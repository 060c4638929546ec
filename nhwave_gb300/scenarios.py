"""Seeded synthetic scenarios in the reference's input formats.

No public benchmark-suite data is used: every input is generated here from a
recorded seed and written in the shapes the reference reads -- ``depth.txt``
(CELL_CENTER: Nglob rows of Mglob values, src/initialize.F:1833-1836),
``eta0.txt`` and ``uvw0.txt`` (src/initialize.F:2994-3017: eta as Nglob rows
of Mglob, then U, V, W each as Kglob x Nglob rows of Mglob).  Arrays returned
here are flat float64 in that order (i fastest).

Workloads (sizes and physics of the five configurations this path is
measured on):
  c1  solitary wave in a flat channel           256 x 8 x 10,   dx=dy=0.1 m
  c2  monochromatic wave over a submerged bar   1024 x 64 x 20, dx=0.025, dy=0.05 m
  c3  rigid submarine landslide, wet/dry beach  512 x 512 x 10, dx=dy=2 m
  c4  ensemble member: random smooth bathymetry, Gaussian hump, walls
plus small versions of each (``tiny_*``) that the CPU oracle runs in seconds.
"""
from __future__ import annotations

import math

import numpy as np

from .params import (
    NHW_FP64, SLIDE_RIGID_3D, WM_INT_LIN, NhwParams, default_params,
)

GRAV = 9.81


def _xc(p: NhwParams) -> np.ndarray:
    return (np.arange(p.Mglob) + 0.5) * p.dx


def _yc(p: NhwParams) -> np.ndarray:
    return (np.arange(p.Nglob) + 0.5) * p.dy


# ------------------------------------------------------------------- c1
def solitary_channel(M=256, N=8, K=10, dx=0.1, h=1.0, amp=0.2, x0=5.0, **kw):
    """KdV solitary wave eta = A sech^2(sqrt(3A/4h^3)(x-x0)), u = sqrt(g/h) eta."""
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dx, dt_ini=0.001, dt_min=1e-6,
                       dt_max=1.0, cfl=0.5, min_dep=0.01, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, sim_steps=1000)
    for k, v in kw.items():
        setattr(p, k, v)
    depth = np.full((N, M), h)
    xs = _xc(p)
    eta1 = amp / np.cosh(math.sqrt(3.0 * amp / (4.0 * h ** 3)) * (xs - x0)) ** 2
    eta = np.broadcast_to(eta1, (N, M)).copy()
    u = math.sqrt(GRAV / h) * eta
    uvw = np.zeros((3, K, N, M))
    uvw[0] = u[None, :, :]
    return p, depth.ravel(), eta.ravel(), uvw.ravel()


# ------------------------------------------------------------------- c2
def bar_depth(x: np.ndarray) -> np.ndarray:
    """Trapezoidal bar: 0.4 m, 1:20 rise over 6-12 m to 0.1 m, flat to 14 m, 1:10 fall to 17 m."""
    d = np.full_like(x, 0.4)
    up = (x > 6.0) & (x <= 12.0)
    d[up] = 0.4 - (x[up] - 6.0) * 0.05
    d[(x > 12.0) & (x <= 14.0)] = 0.1
    dn = (x > 14.0) & (x < 17.0)
    d[dn] = 0.1 + (x[dn] - 14.0) * 0.1
    return d


def submerged_bar(M=1024, N=64, K=20, dx=0.025, dy=0.05, **kw):
    """Internal wavemaker INT_LIN (T=2.02 s, a=0.01 m, h=0.4 m) and 2 m sponges at both ends."""
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.001, dt_min=1e-6,
                       dt_max=1.0, cfl=0.5, min_dep=0.001, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, total_time=20.0)
    p.wavemaker = WM_INT_LIN
    p.amp_wave, p.per_wave, p.dep_wave, p.theta_wave, p.cur_wave = 0.01, 2.02, 0.4, 0.0, 0.0
    p.xsource_west, p.xsource_east = 4.0, 4.2
    p.ysource_suth, p.ysource_nrth = 0.0, N * dy
    p.sponge_on = 1
    p.sponge_west_width = p.sponge_east_width = 2.0
    for k, v in kw.items():
        setattr(p, k, v)
    xs = _xc(p) * (25.6 / (M * dx))  # keep the bar's shape on smaller grids
    depth = np.broadcast_to(bar_depth(xs), (N, M)).copy()
    return p, depth.ravel(), None, None


# ------------------------------------------------------------------- c3
def landslide_beach(M=512, N=512, K=10, dx=2.0, **kw):
    """Plane beach h = 60 - x/15 (dry land past x = 900 m) with a RIGID_3D slide."""
    L = M * dx
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dx, dt_ini=0.01, dt_min=1e-6,
                       dt_max=5.0, cfl=0.5, min_dep=0.01, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, total_time=200.0)
    p.slide_type = SLIDE_RIGID_3D
    p.slide_t, p.slide_l, p.slide_w = 8.0, 100.0 * L / 1024.0, 100.0 * L / 1024.0
    p.slide_ut, p.slide_a0 = 15.0, 0.75            # s0 = ut^2/a0 = 300 m, t0 = ut/a0 = 20 s
    p.slope_angle = math.degrees(math.atan(1.0 / 15.0))
    p.slide_angle = 180.0                            # moving towards deep water (-x)
    p.slide_x0, p.slide_y0 = 0.6 * L, 0.5 * N * dx
    # the Froude cap of the reference's own landslide benchmark input (10);
    # with 100, the thin layers of the runup reach several hundred m/s and
    # dt falls below 2 ms about 44 s into the run
    p.froude_cap = 10.0
    for k, v in kw.items():
        setattr(p, k, v)
    xs = _xc(p) * (1024.0 / L)
    depth = np.broadcast_to(60.0 - xs / 15.0, (N, M)).copy()
    return p, depth.ravel(), None, None


# ------------------------------------------------------------------- c4
def ensemble_member(rng: np.random.Generator, Kchoices=(5, 10, 15, 20), side=(64, 512),
                    dxr=(1.0, 20.0), **kw):
    """One scenario of the uneven ensemble: sides log-uniform in ``side``, K from
    ``Kchoices``, dx log-uniform in ``dxr``; Gaussian-filtered white-noise
    bathymetry (correlation length 20 cells) scaled to 5-200 m; Gaussian eta hump
    of amplitude U[0.01,0.1]*h_local and width 10-40 cells; at rest; walls."""
    from scipy.ndimage import gaussian_filter

    lo, hi = math.log(side[0]), math.log(side[1])
    M = int(round(math.exp(rng.uniform(lo, hi))))
    N = int(round(math.exp(rng.uniform(lo, hi))))
    K = int(rng.choice(Kchoices))
    dx = float(math.exp(rng.uniform(math.log(dxr[0]), math.log(dxr[1]))))
    noise = rng.standard_normal((N, M))
    f = gaussian_filter(noise, sigma=20.0 / 2.0, mode="reflect")
    f = (f - f.min()) / max(f.max() - f.min(), 1e-30)
    depth = 5.0 + 195.0 * f
    ci, cj = rng.uniform(0.25, 0.75) * M, rng.uniform(0.25, 0.75) * N
    h_loc = float(depth[min(int(cj), N - 1), min(int(ci), M - 1)])
    amp = rng.uniform(0.01, 0.1) * h_loc
    width = rng.uniform(10.0, 40.0)
    ii, jj = np.meshgrid(np.arange(M) + 0.5, np.arange(N) + 0.5)
    eta = amp * np.exp(-((ii - ci) ** 2 + (jj - cj) ** 2) / width ** 2)
    c = math.sqrt(GRAV * 200.0)
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dx, dt_ini=0.4 * dx / c,
                       dt_min=1e-8, dt_max=60.0, cfl=0.5, min_dep=0.01, non_hydro=1,
                       time_order=3, tol=1e-8, itmax=1000, sim_steps=500)
    for k, v in kw.items():
        setattr(p, k, v)
    return p, depth.ravel(), eta.ravel(), np.zeros(3 * K * N * M)


def ensemble(n: int, seed: int = 2024, **kw):
    rng = np.random.default_rng(seed)
    return [ensemble_member(rng, **kw) for _ in range(n)]


# --------------------------------------------------------- wave flume
def wave_flume(kind: str = "LIN", M=256, N=4, K=10, dx=0.05, dy=0.05, depth=0.5, amp=0.02, per=1.5,
               sponge=2.0, **kw):
    """Flat flume fed through its west boundary (BC_X0 = 3): a linear wave
    (LEF_LIN, amplitude `amp`, period `per`), a solitary wave (LEF_SOL,
    height `amp`), a second-order Stokes wave (LEF_STK, amplitude `amp`), a
    cnoidal wave (LEF_CON, height `amp`) or a linear wave on a current
    (WAV_CUR, `cur_wave`, `tramp`) or a focused group (FOCUSED, `nwave` ...);
    sponge layer and wall at the east end,
    walls along the sides; at rest initially."""
    from .params import (WM_FOCUSED, WM_LEF_CON, WM_LEF_JON, WM_LEF_LIN, WM_LEF_SOL, WM_LEF_SPC, WM_LEF_STK,
                         WM_LEF_TID, WM_LEF_TMA, WM_WAV_CUR)
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.1 * dx / math.sqrt(GRAV * depth),
                       dt_min=1e-8, dt_max=1.0, cfl=0.5, min_dep=0.001, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, total_time=20.0)
    p.bc_x0 = 3
    p.wavemaker = {"LIN": WM_LEF_LIN, "SOL": WM_LEF_SOL, "STK": WM_LEF_STK, "CON": WM_LEF_CON,
                   "CUR": WM_WAV_CUR, "FOC": WM_FOCUSED, "TID": WM_LEF_TID, "JON": WM_LEF_JON, "TMA": WM_LEF_TMA,
                   "SPC": WM_LEF_SPC}[kind]
    p.amp_wave, p.per_wave, p.dep_wave, p.theta_wave = amp, per, depth, 0.0
    p.sponge_on = 1
    p.sponge_east_width = sponge
    for k, v in kw.items():
        setattr(p, k, v)
    return p, np.full(M * N, depth), None, None


# ------------------------------------------------------ 2-D spectrum
def spc_spectrum(nf: int = 8, nd: int = 3, hm0: float = 0.03, fp: float = 0.7, spread_deg: float = 20.0):
    """A 2-D spectrum for LEF_SPC in spc2d.txt's order (freq [nf], dire [nd],
    densities flat with direction fastest): a JONSWAP-shaped frequency
    spectrum over 0.5-1.2 Hz times a cos^2 spreading over +-spread_deg,
    scaled so that sum S df dtheta = hm0^2/16 with the reference's
    centred band widths."""
    freq = np.linspace(0.5, 1.2, nf)
    dire = np.linspace(-spread_deg, spread_deg, nd)
    sf = freq ** -5 * np.exp(-1.25 * (fp / freq) ** 4) * 3.3 ** np.exp(-0.5 * ((freq / fp - 1) / 0.08) ** 2)
    sd = np.cos(np.radians(dire) * 90.0 / (spread_deg * 1.5)) ** 2
    spc = np.outer(sf, sd)                 # [nf][nd]: direction fastest when flattened

    def widths(a):
        w = np.empty_like(a)
        w[0], w[-1] = a[1] - a[0], a[-1] - a[-2]
        w[1:-1] = 0.5 * (a[2:] - a[:-2])
        return np.abs(w)
    m0 = float((spc * np.outer(widths(freq), widths(dire))).sum())
    spc *= hm0 ** 2 / 16.0 / m0
    return freq, dire, spc.ravel()


# ------------------------------------------------- internal sources
def internal_flume(kind: str = "CON", M=64, N=16, K=5, dx=0.1, dy=0.25, depth=0.5, amp=0.1, per=3.0, **kw):
    """Flat basin with an internal source strip across it at x = 3.0-3.2 m
    and 1.5 m sponges at both ends, walls along the sides, at rest: a
    cnoidal wave (INT_CON, height `amp`, period `per`), the components of a
    JONSWAP or TMA spectrum (INT_JON / INT_TMA: Hm0 3 cm, Tp 1.5 s, 24
    components over 0.4-1.2 Hz), or of a 2-D spectrum (INT_SPC, densities)
    or of given amplitudes and phases (INT_IRR), both passed with
    set_wave_spectrum.  The channel, 4 m wide, repeats cross-channel wave
    numbers of 2 pi / 4 m, to which the spectral makers snap their
    directions."""
    from .params import WM_INT_CON, WM_INT_IRR, WM_INT_JON, WM_INT_SPC, WM_INT_TMA
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.1 * dx / math.sqrt(GRAV * depth),
                       dt_min=1e-8, dt_max=1.0, cfl=0.5, min_dep=0.001, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, total_time=20.0)
    p.wavemaker = {"CON": WM_INT_CON, "JON": WM_INT_JON, "TMA": WM_INT_TMA, "SPC": WM_INT_SPC,
                   "IRR": WM_INT_IRR}[kind]
    p.amp_wave, p.per_wave, p.dep_wave, p.theta_wave = amp, per, depth, 0.0
    p.xsource_west, p.xsource_east = 3.0, 3.2
    p.ysource_suth, p.ysource_nrth = 0.0, N * dy
    if kind in ("JON", "TMA"):
        p.hm0, p.tp, p.freq_min, p.freq_max, p.numfreq, p.wave_seed = 0.03, 1.5, 0.4, 1.2, 24, 11
    p.sponge_on = 1
    p.sponge_west_width = p.sponge_east_width = 1.5
    for k, v in kw.items():
        setattr(p, k, v)
    return p, np.full(M * N, depth), None, None


def irr_components(nf: int = 6, nd: int = 4, amp: float = 0.004, seed: int = 5):
    """Component data of INT_IRR in irr2d.txt's order: nf frequencies over
    0.5-1.2 Hz, nd directions over -30..30 degrees, amplitudes (`amp` over
    the component count, tapered across the band) and seeded phases, flat
    with direction fastest."""
    rng = np.random.default_rng(seed)
    freq = np.linspace(0.5, 1.2, nf)
    dire = np.linspace(-30.0, 30.0, nd)
    a = amp / (nf * nd) * np.outer(np.hanning(nf + 2)[1:-1], np.ones(nd)) * 4.0
    return freq, dire, a.ravel(), rng.uniform(0.0, 2.0 * np.pi, nf * nd)


# ------------------------------------------------------- east inflows
def east_flume(kind: str = "RIG", M=64, N=4, K=5, dx=0.1, dy=0.1, depth=0.5, amp=0.02, per=1.5, **kw):
    """Flumes whose east side is open to a boundary condition (BC_Xn = 3).
    ``RIG``: a linear wave given to the east side (RIG_LIN, amplitude `amp`,
    period `per`), wall and a 1.5 m sponge at the west end.  ``FLR``: the
    FLUX_LR current, in through the west side (BC_X0 = 3) over a smooth bump
    of a fifth of the depth, out through the east side, ramped up over TRAMP
    = 1 s, roughness Zob = 1 mm.  At rest initially."""
    from .params import WM_FLUX_LR, WM_RIG_LIN
    p = default_params(Mglob=M, Nglob=N, Kglob=K, dx=dx, dy=dy, dt_ini=0.1 * dx / math.sqrt(GRAV * depth),
                       dt_min=1e-8, dt_max=1.0, cfl=0.5, min_dep=0.001, non_hydro=1, time_order=3,
                       tol=1e-8, itmax=1000, total_time=20.0)
    p.bc_xn = 3
    p.amp_wave, p.per_wave, p.dep_wave, p.theta_wave = amp, per, depth, 0.0
    xs = _xc(p)
    h = np.full(M, depth)
    if kind == "RIG":
        p.wavemaker = WM_RIG_LIN
        p.sponge_on = 1
        p.sponge_west_width = 1.5
    else:
        p.wavemaker = WM_FLUX_LR
        p.bc_x0 = 3
        p.tramp = 1.0
        p.zob = 1e-3
        h = depth - 0.2 * depth * np.exp(-((xs - 0.5 * M * dx) / (0.1 * M * dx)) ** 2)
    for k, v in kw.items():
        setattr(p, k, v)
    return p, np.broadcast_to(h, (N, M)).copy().ravel(), None, None


# ------------------------------------------------------------ registry
def make(name: str, precision: int = NHW_FP64, seed: int = 0, **kw):
    """Return ``(params, depth, eta0, uvw0)`` for a named scenario."""
    if name == "c1":
        out = solitary_channel(**kw)
    elif name == "c2":
        out = submerged_bar(**kw)
    elif name == "c3":
        out = landslide_beach(**kw)
    elif name == "c4":
        out = ensemble_member(np.random.default_rng(seed), **kw)
    elif name == "tiny_c1":
        out = solitary_channel(M=48, N=4, K=5, x0=1.5, amp=0.1, **kw)
    elif name == "tiny_c2":
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_c3":
        out = landslide_beach(M=48, N=40, K=5, dx=2.0 * 1024 / 48 / 2, **kw)
    elif name == "tiny_c4":
        out = ensemble_member(np.random.default_rng(seed), Kchoices=(4, 5), side=(24, 48), **kw)
    elif name == "tiny_flume_lin":
        out = wave_flume("LIN", M=64, N=4, K=5, dx=0.1, dy=0.1, sponge=1.5, **kw)
    elif name == "tiny_flume_sol":
        out = wave_flume("SOL", M=64, N=4, K=5, dx=0.1, dy=0.1, amp=0.05, sponge=1.5, **kw)
    elif name == "tiny_flume_stk":
        out = wave_flume("STK", M=64, N=4, K=5, dx=0.1, dy=0.1, amp=0.04, per=1.5, sponge=1.5, **kw)
    elif name == "tiny_flume_con":
        # Ursell number H L^2 / h^3 of about 34: elliptic parameter m = 0.91
        out = wave_flume("CON", M=64, N=4, K=5, dx=0.1, dy=0.1, amp=0.1, per=3.0, sponge=1.5, **kw)
    elif name == "tiny_visc":
        # the small submerged bar with constant viscosities (VISCOUS_FLOW, IVTURB = IHTURB = 1)
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.005, chs=0.01), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_visc_dt":
        # as tiny_visc, with a horizontal viscosity large enough that VISCOUS_NUMBER limits dt
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.05, chs=20.0), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_visc_noslip":
        # tiny_visc on a no-slip bed (BC_Z0 = 2)
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.005, chs=0.01, bc_z0=2), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_visc_fric":
        # tiny_visc with the friction law on the bed (BC_Z0 = 5) and on the south, north and east
        # walls (BC = 5), from a drag coefficient (Ibot = 1)
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.005, chs=0.01, bc_z0=5, bc_y0=5, bc_yn=5, bc_xn=5,
                       ibot=1, cd0=0.006), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_visc_sgs":
        # the small submerged bar with the subgrid eddy viscosities (IVTURB = IHTURB = 2)
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.2, chs=0.2, ivturb=2, ihturb=2), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_visc_sgs_fric":
        # tiny_visc_sgs with the friction law on the bed and on the south, north and east walls
        kw = dict(dict(viscous_flow=1, visc=1e-6, cvs=0.2, chs=0.2, ivturb=2, ihturb=2, bc_z0=5, bc_y0=5,
                       bc_yn=5, bc_xn=5, ibot=1, cd0=0.006), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_ke":
        # the small submerged bar with the 3-D k-epsilon closure (IVTURB = IHTURB = 10, PRODTYPE 3)
        # on a friction-law bed; tests seed tke and epsilon above their floors
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=10, ihturb=10, prod_type=3, bc_z0=5, ibot=1, cd0=0.006),
                  **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_ke_rng":
        # tiny_ke with the RNG variant, vertical-shear production (PRODTYPE 2) and friction
        # walls (BC = 5) on the south, north and east sides with a roughness height (Ibot = 2)
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=10, ihturb=10, rng=1, prod_type=2, bc_z0=5, bc_y0=5,
                       bc_yn=5, bc_xn=5, ibot=2, zob=1e-3), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_ke2":
        # the small submerged bar with the 2-D k-epsilon closure (IVTURB = 3, CmuHt = CmuVt); tests seed
        # tke and epsilon above their floors
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=3, ihturb=10), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_flume_ke2":
        # the linear-wave flume (LEF_LIN) with the 2-D k-epsilon closure, whose first six columns
        # stay at the floors
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=3, ihturb=1, chs=0.001), **kw)
        out = wave_flume("LIN", M=64, N=4, K=5, dx=0.1, dy=0.1, sponge=1.5, **kw)
    elif name == "tiny_lesdyn":
        # the small submerged bar with the dynamic Smagorinsky LES (IVTURB = 30, CmuHt = CmuVt)
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=30, ihturb=30), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_les":
        # the small submerged bar with the Smagorinsky LES closure (IVTURB = 20, CmuHt = CmuVt)
        kw = dict(dict(viscous_flow=1, visc=1e-6, ivturb=20, ihturb=20, cvs=0.1), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_fric_log":
        # the inviscid small bar with the friction law on the bed and the side walls, from a
        # roughness height (Ibot = 2)
        kw = dict(dict(bc_z0=5, bc_y0=5, bc_yn=5, bc_xn=5, ibot=2, zob=1e-3), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_wallfric":
        # the inviscid small bar with wall friction (BC = 5) on every side, drag coefficient 0.01
        kw = dict(dict(bc_x0=5, bc_xn=5, bc_y0=5, bc_yn=5, ibot=1, cd0=0.01), **kw)
        out = submerged_bar(M=96, N=6, K=6, dx=25.6 / 96, dy=0.2, **kw)
    elif name == "tiny_flume_tid":
        # the S2 tide (LEF_TID) of 0.1 m amplitude from its zero crossing
        out = wave_flume("TID", M=64, N=4, K=5, dx=0.1, dy=0.1, amp=0.1, sponge=1.5, **kw)
    elif name == "tiny_flume_foc":
        # a focused group of 8 components around 1 Hz (FOCUSED), focusing 3 m in at t = 4 s
        kw = dict(dict(nwave=8, component_amp_type=2, f_center=1.0, normalized_delta_f=0.6, x_breaking=3.0,
                       t_breaking=4.0, slope_group=0.25, depth_comp=0.5), **kw)
        out = wave_flume("FOC", M=64, N=4, K=5, dx=0.1, dy=0.1, sponge=1.5, **kw)
    elif name == "tiny_flume_cur":
        # LEF_LIN on a current of 0.05 m/s ramped up over TRAMP = 0.5 s (WAV_CUR), out at an Orlanski east side
        kw = dict(dict(cur_wave=0.05, tramp=0.5, bc_xn=6, sponge_on=0), **kw)
        out = wave_flume("CUR", M=64, N=4, K=5, dx=0.1, dy=0.1, **kw)
    elif name == "tiny_open":
        # solitary wave whose front already touches an open (Orlanski, BC_Xn = 6) east side
        out = solitary_channel(M=48, N=4, K=5, x0=3.0, amp=0.1, bc_xn=6, **kw)
    elif name in ("tiny_flume_jon", "tiny_flume_tma"):
        # irregular waves of a JONSWAP (TMA) spectrum, Hm0 3 cm, Tp 1.5 s, 24 components over 0.4-1.2 Hz
        kw = dict(dict(hm0=0.03, tp=1.5, freq_min=0.4, freq_max=1.2, numfreq=24, wave_seed=11), **kw)
        out = wave_flume(name[-3:].upper(), M=64, N=4, K=5, dx=0.1, dy=0.1, sponge=1.5, **kw)
    elif name == "tiny_flume_spc":
        # directional irregular waves from a 2-D spectrum (LEF_SPC; the spectrum itself is
        # scenarios.spc_spectrum(), passed with set_wave_spectrum); 8 cross-channel rows
        out = wave_flume("SPC", M=64, N=8, K=5, dx=0.1, dy=0.1, sponge=1.5, **kw)
    elif name in ("tiny_int_con", "tiny_int_jon", "tiny_int_tma", "tiny_int_spc", "tiny_int_irr"):
        # the internal source strip of each spectral or cnoidal maker; INT_SPC's spectrum is
        # spc_spectrum(8, 5, spread_deg=30), INT_IRR's components irr_components()
        amp = 0.1 if name.endswith("con") else 0.0
        out = internal_flume(name[-3:].upper(), amp=amp, **kw)
    elif name == "tiny_flume_rig":
        # a linear wave given to the east side (RIG_LIN through BC_Xn = 3), wall and sponge at the west
        out = east_flume("RIG", **kw)
    elif name == "tiny_flux_lr":
        # the FLUX_LR current through the west (BC_X0 = 3) and east (BC_Xn = 3) sides, over a bump
        out = east_flume("FLR", depth=0.3, **kw)
    elif name == "tiny_flume_open":
        # linear wave fed in at the west and let out through an Orlanski east side, no sponge
        out = wave_flume("LIN", M=64, N=4, K=5, dx=0.1, dy=0.1, bc_xn=6, sponge_on=0, **kw)
    else:
        raise KeyError(name)
    p = out[0]
    p.precision = precision
    return out


def cell_updates(p: NhwParams, steps: int) -> int:
    return int(p.Mglob) * int(p.Nglob) * int(p.Kglob) * int(steps)
