"""GPU parity: the C-ABI library against the CPU oracle on the same seeded inputs.

Bars (FP64 form): masks bit-exact; set-up and the explicit routines bit-exact
(the FP64 kernels are built without FMA contraction and follow the reference's
evaluation order); after full steps, whose Poisson solves differ only by the
solver's stopping point, eta/U/V/W/P within 1e-10 relative L2 with TOL=1e-12.
FP32+IR form: eta within 1e-6 relative L2 of the FP64 oracle, masks bit-exact.
"""
import numpy as np
import pytest

from conftest import rel_l2, seed_ke

pytestmark = pytest.mark.gpu

CASES = ["tiny_c1", "tiny_c2", "tiny_c3", "tiny_c4"]
# plus a solitary wave leaving through an open (Orlanski, BC_Xn = 6) east
# side, and the small submerged bar with constant viscosities (VISCOUS_FLOW;
# in tiny_visc_dt the viscous limit sets dt; no-slip and friction-law beds;
# the subgrid eddy viscosities, IVTURB = IHTURB = 2; the k-epsilon closure,
# IVTURB = IHTURB = 10, standard and RNG, and the 2-D one, IVTURB = 3, from
# seeded turbulence; the Smagorinsky and dynamic LES, IVTURB = 20 and 30),
# and wall friction (BC = 5) on the sides
MORE_CASES = CASES + ["tiny_open", "tiny_visc", "tiny_visc_dt", "tiny_visc_noslip", "tiny_visc_fric",
                      "tiny_visc_sgs", "tiny_visc_sgs_fric", "tiny_ke", "tiny_ke_rng", "tiny_ke2", "tiny_flume_ke2",
                      "tiny_les", "tiny_lesdyn", "tiny_wallfric"]
STATE2D = ["D", "ETA", "HC", "HFX0", "HFY0", "DELXH", "DELYH", "ETAXL", "ETAXR", "ETAYL", "ETAYR"]
STATE3D = ["U", "V", "W", "DU", "DV", "DW"]


def vel_err(g, o, name):
    """Error of one velocity component relative to the whole velocity field
    (a component that is zero up to roundoff has no relative error of its own)."""
    from nhwave_gb300 import fields as F
    fid = getattr(F, name)
    sl = o.shape.interior(fid)
    ref = np.sqrt(sum(np.linalg.norm(o.get(getattr(F, c))[sl]) ** 2 for c in ("U", "V", "W")))
    return np.linalg.norm(g.get(fid)[sl] - o.get(fid)[sl]) / ref


# Poisson TOL of the step tests: 1e-13 sits above the FP64 residual floor
# (about 1e-14 on these grids), so both solvers stop by convergence
STEP_TOL = 1e-13


def _pair(name, oracle_mod, precision=0, tol=STEP_TOL, seed=7, **kw):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=precision, seed=seed, **kw)
    p.tol = tol
    p.itmax = 20000
    g = lib.Scenario(p, d, e, u)
    q = p.copy()
    q.precision = 0
    o = oracle_mod.Oracle(q, d, e, u)
    if p.viscous_flow and p.ivturb in (3, 10):
        seed_ke(g, o)
    return g, o


def _cmp_exact(g, o, names, where):
    from nhwave_gb300 import fields as F
    for n in names:
        fid = getattr(F, n)
        a, b = g.get(fid), o.get(fid)
        sl = o.shape.interior(fid) if n in ("HFX0", "HFY0", "DELXH", "DELYH") else Ellipsis
        bad = np.argwhere(a[sl] != b[sl])
        assert bad.size == 0, f"{where}: {n} differs at {bad[:5].tolist()} (max |d| {np.abs(a[sl]-b[sl]).max():.3e})"


@pytest.mark.parametrize("name", CASES)
def test_setup_bit_exact(name, oracle_mod, gpu_lib):
    g, o = _pair(name, oracle_mod)
    _cmp_exact(g, o, ["MASK", "MASK_STRUCT", "MASK9"] + STATE2D + ["SPONGE"] + STATE3D, "setup")


@pytest.mark.parametrize("hllc", [0, 1])
@pytest.mark.parametrize("name", MORE_CASES)
def test_explicit_routines_bit_exact(name, hllc, oracle_mod, gpu_lib):
    """estimate_dt .. fluxes, and a hydrostatic eval_duvw, match operation for
    operation, with HLL and with HLLC face fluxes (src/nhwave.F:1705-1709)."""
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod, non_hydro=0, hllc=hllc)
    for rnd in range(2):
        for obj in (g, o):
            assert obj.estimate_dt() == 0
            if obj.params.slide_type:
                obj.update_bathymetry()
            obj.update_mask()
            obj.update_vars()
        sg, so = g.scalars(), o.scalars()
        assert sg.dt == so.dt and sg.time == so.time and sg.run_step == so.run_step
        if g.params.slide_type:
            # the slide shape uses cosh/log: CUDA's and the host libm's may differ
            # in the last bit, so compare with a tolerance and pin the inputs
            for n in ("HC", "HFX", "HFY", "HFX0", "HFY0", "DELXH", "DELYH", "DELTH", "DELT2H"):
                fid = getattr(F, n)
                sl = o.shape.interior(fid)
                # DeltH = (Hc - Ho)/dt amplifies last-bit differences of Hc
                lim = 1e-8 if n in ("DELTH", "DELT2H") else 1e-13
                r = rel_l2(g.get(fid)[sl], o.get(fid)[sl])
                assert r < lim, f"{n} after update_bathymetry: {r:.3e}"
                g.set(fid, o.get(fid))
        _cmp_exact(g, o, ["MASK", "MASK9", "D", "ETA", "HC", "DELXH", "DELYH"], f"prologue {rnd}")
        for s in range(1, 4):
            g.source_terms(); o.source_terms()
            _cmp_exact(g, o, ["SOURCEX", "SOURCEY"], f"source_terms {rnd}.{s}")
            sc = rel_l2(g.get(F.SOURCEC), o.get(F.SOURCEC))
            assert sc < 1e-14, f"SourceC rel {sc}"
            g.set(F.SOURCEC, o.get(F.SOURCEC))  # cos() of CUDA vs libm: pin the input
            g.fluxes(); o.fluxes()
            sl = o.shape.interior
            for n in ("EX", "FX", "GX", "HX", "EY", "FY", "GY", "HY", "FZ", "GZ", "HZ"):
                fid = getattr(F, n)
                a, b = g.get(fid)[sl(fid)], o.get(fid)[sl(fid)]
                assert np.array_equal(a, b), f"fluxes {rnd}.{s}: {n} max |d| {np.abs(a-b).max():.3e}"
            g.eval_duvw(s); o.eval_duvw(s)
            _cmp_exact(g, o, ["D", "ETA", "MASK", "R1", "DELXETA", "DELYETA"] + STATE3D, f"eval_duvw {rnd}.{s}")
            a, b = g.get(F.OMEGA), o.get(F.OMEGA)
            assert np.array_equal(a, b), f"omega max |d| {np.abs(a-b).max():.3e}"
            if g.params.sponge_on:
                g.sponge_damping(); o.sponge_damping()
                _cmp_exact(g, o, ["D", "ETA"] + STATE3D, f"sponge {rnd}.{s}")
            if g.params.viscous_flow:
                g.eval_turb(s); o.eval_turb(s)
                if g.params.ivturb in (20, 30):
                    # the LES filter width and wall function use pow/log/exp: CUDA's
                    # and the host libm's may differ in the last bit; pin after
                    for n in ("CMUVT", "CMUHT"):
                        fid = getattr(F, n)
                        r = rel_l2(g.get(fid), o.get(fid))
                        assert r < 1e-13, f"eval_turb {rnd}.{s}: {n} rel {r:.3e}"
                        g.set(fid, o.get(fid))
                ke = ["TKE", "EPS", "DTKE", "DEPS"] if g.params.ivturb in (3, 10) else []
                _cmp_exact(g, o, ["CMUVT", "CMUHT"] + ke, f"eval_turb {rnd}.{s}")
    g.close()


BATHY = ("HC", "HFX", "HFY", "HFX0", "HFY0", "DELXH", "DELYH", "DELTH", "DELT2H")
# The moving slide's bed depends on cosh/log of CUDA (device) and of the host
# libm (oracle); their last-bit differences are amplified by the second time
# difference Delt2H = (DeltH - DeltHo)/dt that forces P at the bed, to ~1e-8
# relative -- a sensitivity of the reference's own scheme to its libm.
SLIDE_TOL = {"ETA": 1e-9, "P": 1e-7, "U": 1e-7, "V": 1e-7, "W": 1e-7}


def step_pinned(g, o):
    """One step routine by routine, copying the oracle's bathymetry after update_bathymetry."""
    from nhwave_gb300 import fields as F
    for obj in (g, o):
        assert obj.estimate_dt() == 0
        obj.update_bathymetry()
    for n in BATHY:
        g.set(getattr(F, n), o.get(getattr(F, n)))
    for obj in (g, o):
        obj.update_mask()
        obj.update_vars()
        for s in range(1, 4):
            obj.source_terms()
            obj.fluxes()
            assert obj.eval_duvw(s) == 0
            if obj.params.sponge_on:
                obj.sponge_damping()
            obj.eval_turb(s)


@pytest.mark.parametrize("name", MORE_CASES)
def test_steps_fp64(name, oracle_mod, gpu_lib):
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod)
    for n in range(6):
        if g.params.slide_type:
            step_pinned(g, o)
        else:
            assert g.step() == 0
            assert o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    for f in ("ETA", "P"):
        fid = getattr(F, f)
        r = rel_l2(g.get(fid)[sl(fid)], o.get(fid)[sl(fid)])
        assert r < 1e-10, f"{name} {f}: rel L2 {r:.3e}"
    for f in ("U", "V", "W"):
        r = vel_err(g, o, f)
        assert r < 1e-10, f"{name} {f}: rel L2 {r:.3e}"
    sg, so = g.scalars(), o.scalars()
    assert abs(sg.time - so.time) <= 1e-12 * so.time
    assert sg.last_rel_residual <= STEP_TOL
    g.close()


def test_slide_free_running(oracle_mod, gpu_lib):
    """The slide case stepped freely on both sides: masks bit-exact, the rest within SLIDE_TOL."""
    from nhwave_gb300 import fields as F
    g, o = _pair("tiny_c3", oracle_mod)
    for n in range(6):
        assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    for f, lim in SLIDE_TOL.items():
        r = vel_err(g, o, f) if f in ("U", "V", "W") else rel_l2(g.get(getattr(F, f))[sl(getattr(F, f))],
                                                                o.get(getattr(F, f))[sl(getattr(F, f))])
        assert r < lim, f"slide {f}: {r:.3e}"
    g.close()


# FP32+IR against the FP64 oracle after 6 steps of the small cases, per field:
# eta relative L2, P relative L2, U/V/W relative to the whole velocity field.
# Largest values measured on a GB300 over these cases: eta 1.5e-8, P 4.1e-6
# (tiny_open), U 1.5e-6 and V 1.5e-6 (tiny_c4), W 2.0e-7; the bounds leave a
# factor of about 5, and eta is held to the 1e-6 the FP32+IR form is built for.
FP32IR_BOUNDS = {"ETA": 1e-6, "P": 2e-5, "U": 1e-5, "V": 1e-5, "W": 2e-6}


@pytest.mark.parametrize("name", MORE_CASES)
def test_steps_fp32_ir(name, oracle_mod, gpu_lib):
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod, precision=1, tol=1e-10)
    eta0 = o.get(F.ETA)[o.shape.interior(F.ETA)].copy()
    for n in range(6):
        assert g.step() == 0
        assert o.step() == 0
    sl = o.shape.interior
    assert np.array_equal(g.get(F.MASK), o.get(F.MASK))
    err = {f: rel_l2(g.get(getattr(F, f))[sl(getattr(F, f))], o.get(getattr(F, f))[sl(getattr(F, f))])
           for f in ("ETA", "P")}
    err.update({f: vel_err(g, o, f) for f in ("U", "V", "W")})
    print(f"\n{name} FP32+IR vs FP64 oracle, 6 steps: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for f, r in err.items():
        assert r < FP32IR_BOUNDS[f], f"{name} {f} rel L2 {r:.3e} (|eta0| {np.abs(eta0).max():.3e})"
    assert g.scalars().last_rel_residual <= 1e-10
    g.close()


@pytest.mark.parametrize("name", CASES)
def test_golden_fixtures(name, gpu_lib):
    import os
    from nhwave_gb300 import fields as F, lib, scenarios as S
    from test_oracle import GOLDEN, golden_path
    steps = GOLDEN[name]
    ref = np.load(golden_path(name, steps))
    p, d, e, u = S.make(name, seed=7)
    p.tol = STEP_TOL
    p.itmax = 20000
    g = lib.Scenario(p, d, e, u)
    for _ in range(steps):
        assert g.step() == 0
    vref = np.sqrt(sum(np.linalg.norm(ref[c]) ** 2 for c in ("U", "V", "W")))
    for f in ("ETA", "D", "U", "V", "W", "P", "OMEGA"):
        fid = getattr(F, f)
        a = g.get(fid)[g.shape.interior(fid)]
        den = vref if f in ("U", "V", "W") else np.linalg.norm(ref[f])
        r = np.linalg.norm(a - ref[f]) / den
        lim = SLIDE_TOL.get(f, 1e-7) if p.slide_type else 1e-10
        assert r < lim, f"{name} {f}: rel L2 {r:.3e}"
    assert np.array_equal(g.get(F.MASK)[g.shape.interior(F.MASK)], ref["MASK"])
    g.close()


# tiny_flume_open: LEF_LIN in at the west, out through an Orlanski east side;
# tiny_flume_stk / _con: second-order Stokes and cnoidal waves fed in
# tiny_flume_rig / tiny_flux_lr: the east side open to RIG_LIN and to the
# FLUX_LR current (BC_Xn = 3)
FLUMES = ["tiny_flume_lin", "tiny_flume_sol", "tiny_flume_stk", "tiny_flume_con", "tiny_flume_open", "tiny_flume_cur",
          "tiny_flume_foc", "tiny_flume_tid", "tiny_flume_rig", "tiny_flux_lr", "tiny_flume_jon", "tiny_flume_tma",
          "tiny_int_con", "tiny_int_jon", "tiny_int_tma",
          "tiny_fric_log"]   # and the friction law from a roughness height: log() of CUDA and libm


@pytest.mark.parametrize("name", FLUMES)
def test_flume_steps_fp64(name, oracle_mod, gpu_lib):
    """Waves fed through the west boundary (BC_X0 = 3, LEF_LIN / LEF_SOL /
    LEF_STK / LEF_CON), one of them leaving through an open east side
    (BC_Xn = 6): FP64 steps against the oracle.  The boundary values use
    cos/sin/cosh/sinh/asin, whose CUDA and host results may differ in the
    last bit, hence 1e-9."""
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod)
    for n in range(20):
        assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    for f in ("ETA", "P"):
        fid = getattr(F, f)
        r = rel_l2(g.get(fid)[sl(fid)], o.get(fid)[sl(fid)])
        assert r < 1e-9, f"{name} {f}: rel L2 {r:.3e}"
    for f in ("U", "W"):
        r = vel_err(g, o, f)
        assert r < 1e-9, f"{name} {f}: {r:.3e}"
    g.close()


@pytest.mark.parametrize("name", FLUMES)
def test_flume_steps_fp32_ir(name, oracle_mod, gpu_lib):
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod, precision=1, tol=1e-10)
    for _ in range(20):
        assert g.step() == 0 and o.step() == 0
    sl = o.shape.interior
    assert np.array_equal(g.get(F.MASK), o.get(F.MASK))
    r = rel_l2(g.get(F.ETA)[sl(F.ETA)], o.get(F.ETA)[sl(F.ETA)])
    assert r < 1e-6, f"{name} eta rel L2 {r:.3e}"
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_hllc_steps(name, precision, oracle_mod, gpu_lib):
    """Whole non-hydrostatic steps with HLLC=T: FP64 within 1e-10 of the
    oracle (eta and P), FP32+IR eta within 1e-6; the mask bit for bit (the
    landslide case has a moving wet/dry front, where the dry-side star
    speeds of src/nhwave.F:2842-2853 are used).  FP64 steps the slide case
    with the oracle's bathymetry pinned, as test_steps_fp64 does."""
    from nhwave_gb300 import fields as F
    g, o = _pair(name, oracle_mod, precision=precision, hllc=1)
    for n in range(6):
        if precision == 0 and g.params.slide_type:
            step_pinned(g, o)
        else:
            assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    lim = 1e-10 if precision == 0 else 1e-6
    r = rel_l2(g.get(F.ETA)[sl(F.ETA)], o.get(F.ETA)[sl(F.ETA)])
    assert r < lim, f"{name} eta rel L2 {r:.3e}"
    if precision == 0:
        r = rel_l2(g.get(F.P)[sl(F.P)], o.get(F.P)[sl(F.P)])
        assert r < 1e-10, f"{name} P rel L2 {r:.3e}"
        for f in ("U", "V", "W"):
            r = vel_err(g, o, f)
            assert r < 1e-10, f"{name} {f}: rel L2 {r:.3e}"
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["tiny_c2", "tiny_c3"])
def test_statistics_like_the_oracle(name, precision, oracle_mod, gpu_lib):
    """nhw_statistics (statistics, src/nhwave.F:3118-3160) against the oracle
    after steps: the GPU sums in a fixed block order, the oracle in the
    reference's loop order, and the fields agree to the solver tolerance."""
    g, o = _pair(name, oracle_mod, precision=precision)
    for _ in range(3):
        assert g.step() == 0 and o.step() == 0
    a, b = g.statistics(), o.statistics()
    lim = 1e-9 if precision == 0 else 1e-5
    for key in ("mass_volume", "energy", "max_eta", "min_eta", "max_u", "max_v", "max_w"):
        # absolute floor: in the nearly 2-D submerged bar |V| is roundoff (~1e-19)
        assert abs(a[key] - b[key]) <= lim * abs(b[key]) + 1e-14, f"{name} {key}: {a[key]!r} vs {b[key]!r}"
    assert a["mass_volume"] == pytest.approx(g.mass(), rel=1e-13)
    g.close()


def test_wave_phases_given_by_the_driver(oracle_mod, gpu_lib):
    """nhw_set_wave_phases: the driver's own phases for the LEF_JON components
    (the reference's RanPhs) replace the seeded ones; GPU and oracle, given the
    same phases, step alike, and differently from the seeded run."""
    from nhwave_gb300 import fields as F
    g, o = _pair("tiny_flume_jon", oracle_mod)
    g2, _ = _pair("tiny_flume_jon", oracle_mod)
    ph = np.random.default_rng(3).uniform(0.0, 2.0 * np.pi, g.params.numfreq)
    g.set_wave_phases(ph)
    o.set_wave_phases(ph)
    for _ in range(10):
        assert g.step() == 0 and o.step() == 0 and g2.step() == 0
    sl = o.shape.interior(F.ETA)
    assert rel_l2(g.get(F.ETA)[sl], o.get(F.ETA)[sl]) < 1e-9
    assert rel_l2(g2.get(F.ETA)[sl], o.get(F.ETA)[sl]) > 1e-3
    from nhwave_gb300 import lib
    with pytest.raises(lib.NhwError):
        g.set_wave_phases(ph[:-1])
    g.close()
    g2.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_spectral_inflow_steps(precision, oracle_mod, gpu_lib):
    """LEF_SPC: directional irregular waves from a 2-D spectrum passed with
    nhw_set_wave_spectrum (seeded phases on both sides); FP64 within 1e-9 of
    the oracle (cos/cosh/tanh of CUDA and libm), FP32+IR eta within 1e-6.
    Before a spectrum is given, update_wave_bc refuses to run."""
    from nhwave_gb300 import fields as F, lib, scenarios as S
    g, o = _pair("tiny_flume_spc", oracle_mod, precision=precision, tol=STEP_TOL if precision == 0 else 1e-10)
    with pytest.raises(lib.NhwError):
        g.update_wave_bc()
    freq, dire, spc = S.spc_spectrum()
    g.set_wave_spectrum(freq, dire, spc)
    o.set_wave_spectrum(freq, dire, spc)
    for n in range(20):
        assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    if precision == 0:
        for f in ("ETA", "P"):
            fid = getattr(F, f)
            r = rel_l2(g.get(fid)[sl(fid)], o.get(fid)[sl(fid)])
            assert r < 1e-9, f"LEF_SPC {f}: rel L2 {r:.3e}"
        for f in ("U", "V", "W"):
            r = vel_err(g, o, f)
            assert r < 1e-9, f"LEF_SPC {f}: {r:.3e}"
    else:
        r = rel_l2(g.get(F.ETA)[sl(F.ETA)], o.get(F.ETA)[sl(F.ETA)])
        assert r < 1e-6, f"LEF_SPC FP32+IR eta rel L2 {r:.3e}"
    # directional: the cross-channel velocity is not zero
    assert np.abs(o.get(F.V)[sl(F.V)]).max() > 1e-5
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kind", ["spc", "irr"])
def test_internal_spectral_source_steps(kind, precision, oracle_mod, gpu_lib):
    """INT_SPC / INT_IRR: the internal source strip fed by a 2-D spectrum (or
    INT_IRR's amplitudes and phases) passed with nhw_set_wave_spectrum, the
    directions snapped to ones the 4 m channel repeats; FP64 within 1e-9 of
    the oracle (cos of CUDA and libm), FP32+IR eta within 1e-6.  Before a
    spectrum is given, source_terms refuses to run; a direction beyond 90
    degrees is refused."""
    from nhwave_gb300 import fields as F, lib, scenarios as S
    g, o = _pair(f"tiny_int_{kind}", oracle_mod, precision=precision, tol=STEP_TOL if precision == 0 else 1e-10)
    with pytest.raises(lib.NhwError):
        g.source_terms()
    if kind == "spc":
        freq, dire, spc = S.spc_spectrum(8, 5, spread_deg=30.0)
        ph = None
        with pytest.raises(lib.NhwError):
            g.set_wave_spectrum(freq, np.array([-30.0, 0.0, 95.0, 10.0, 20.0]), spc)
    else:
        freq, dire, spc, ph = S.irr_components()
        with pytest.raises(lib.NhwError):   # INT_IRR's phases are part of its data
            g.set_wave_spectrum(freq, dire, spc)
    g.set_wave_spectrum(freq, dire, spc, ph)
    o.set_wave_spectrum(freq, dire, spc, ph)
    for n in range(20):
        assert g.step() == 0 and o.step() == 0
        assert np.array_equal(g.get(F.MASK), o.get(F.MASK)), f"mask differs after step {n}"
    sl = o.shape.interior
    if precision == 0:
        for f in ("ETA", "P"):
            fid = getattr(F, f)
            r = rel_l2(g.get(fid)[sl(fid)], o.get(fid)[sl(fid)])
            assert r < 1e-9, f"INT_{kind.upper()} {f}: rel L2 {r:.3e}"
        for f in ("U", "V", "W"):
            r = vel_err(g, o, f)
            assert r < 1e-9, f"INT_{kind.upper()} {f}: {r:.3e}"
        r = rel_l2(g.get(F.SOURCEC)[sl(F.SOURCEC)], o.get(F.SOURCEC)[sl(F.SOURCEC)])
        assert r < 1e-10, f"INT_{kind.upper()} SourceC: rel L2 {r:.3e}"
    else:
        r = rel_l2(g.get(F.ETA)[sl(F.ETA)], o.get(F.ETA)[sl(F.ETA)])
        assert r < 1e-6, f"INT_{kind.upper()} FP32+IR eta rel L2 {r:.3e}"
    # the snapped directions give a cross-channel flow
    assert np.abs(o.get(F.V)[sl(F.V)]).max() > 1e-6
    g.close()


def test_internal_jonswap_phases_given_by_the_driver(oracle_mod, gpu_lib):
    """nhw_set_wave_phases on INT_JON: GPU and oracle, given the same phases,
    step alike, and differently from the seeded run."""
    from nhwave_gb300 import fields as F
    g, o = _pair("tiny_int_jon", oracle_mod)
    g2, _ = _pair("tiny_int_jon", oracle_mod)
    ph = np.random.default_rng(8).uniform(0.0, 2.0 * np.pi, g.params.numfreq)
    g.set_wave_phases(ph)
    o.set_wave_phases(ph)
    for _ in range(10):
        assert g.step() == 0 and o.step() == 0 and g2.step() == 0
    sl = o.shape.interior(F.ETA)
    assert rel_l2(g.get(F.ETA)[sl], o.get(F.ETA)[sl]) < 1e-9
    assert rel_l2(g2.get(F.ETA)[sl], o.get(F.ETA)[sl]) > 1e-3
    g.close()
    g2.close()
