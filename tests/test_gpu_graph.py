"""GPU: the captured step graph (device-side refinement and iteration loops)
against the same routines launched one by one through the C interface.

Both paths run the same kernels in the same order on the same data, so every
field must agree bit for bit, in both precisions.  Also checks the device-side
run gate of nhw_run (TOTAL_TIME / SIM_STEPS) and the solver counters.
"""
import numpy as np
import pytest

from conftest import seed_ke

pytestmark = pytest.mark.gpu

FIELDS = ["D", "ETA", "HC", "U", "V", "W", "DU", "DV", "DW", "P", "OMEGA", "MASK"]


def _scen(name, precision, **attrs):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=precision, seed=11)
    p.tol = 1e-10 if precision == 0 else 1e-8
    p.itmax = 5000
    for k, v in attrs.items():
        setattr(p, k, v)
    s = lib.Scenario(p, d, e, u)
    if p.viscous_flow and p.ivturb in (3, 10):
        seed_ke(s)
    return s


def _routines(s):
    """One time step as the reference's main loop calls it (src/nhwave.F:119-200)."""
    s.estimate_dt()
    if s.params.slide_type:
        s.update_bathymetry()
    s.update_wave_bc()
    s.update_mask()
    s.update_vars()
    for st in range(1, int(s.params.time_order) + 1):
        s.source_terms()
        s.fluxes()
        s.eval_duvw(st)
        if s.params.sponge_on:
            s.sponge_damping()
        s.eval_turb(st)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["tiny_c1", "tiny_c2", "tiny_c3", "tiny_c4", "tiny_flume_lin", "tiny_flume_sol",
                                  "tiny_flume_stk", "tiny_flume_con", "tiny_flume_cur", "tiny_flume_foc", "tiny_flume_tid", "tiny_open",
                                  "tiny_flume_open", "tiny_flume_rig", "tiny_flux_lr", "tiny_flume_jon",
                                  "tiny_visc", "tiny_visc_fric", "tiny_visc_sgs_fric", "tiny_ke", "tiny_ke_rng",
                                  "tiny_les", "tiny_lesdyn", "tiny_ke2", "tiny_flume_ke2"])
def test_graph_step_equals_routines(name, precision, gpu_lib, hllc=0):
    from nhwave_gb300 import fields as F
    a = _scen(name, precision, hllc=hllc)
    b = _scen(name, precision, hllc=hllc)
    for n in range(3):
        a.step()
        _routines(b)
        sa, sb = a.scalars(), b.scalars()
        assert (sa.time, sa.dt, sa.run_step) == (sb.time, sb.dt, sb.run_step)
        assert sa.total_krylov_iters == sb.total_krylov_iters
        assert sa.poisson_solves == sb.poisson_solves
        ke = ["TKE", "EPS", "CMUVT", "CMUHT"] if a.params.viscous_flow and a.params.ivturb in (3, 10) else []
        for f in FIELDS + ke:
            fid = getattr(F, f)
            x, y = a.get(fid), b.get(fid)
            bad = np.argwhere(x != y)
            assert bad.size == 0, f"step {n}: {f} differs at {bad[:4].tolist()}"


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["tiny_c2", "tiny_c3"])
def test_graph_step_equals_routines_hllc(name, precision, gpu_lib):
    """The same with HLLC=T face fluxes."""
    test_graph_step_equals_routines(name, precision, gpu_lib, hllc=1)


def test_run_gate_sim_steps(gpu_lib):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make("tiny_c1", precision=1, seed=11)
    p.sim_steps = 5
    p.total_time = 1e9
    s = lib.Scenario(p, d, e, u)
    assert s.run(40) == 5
    assert s.scalars().run_step == 5
    assert s.run(10) == 0          # the gate stays shut
    assert s.scalars().run_step == 5


def test_run_gate_total_time(gpu_lib):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make("tiny_c2", precision=1, seed=11)
    p.sim_steps = 100000
    s0 = lib.Scenario(p, d, e, u)
    s0.step()
    dt = s0.scalars().dt
    p.total_time = 3.5 * dt        # dt grows at most by 5 % a step
    s = lib.Scenario(p, d, e, u)
    done = s.run(50)
    sc = s.scalars()
    assert 2 <= done <= 4 and sc.run_step == done
    assert sc.time >= p.total_time
    # the same steps one call at a time stop at the same point
    r = lib.Scenario(p, d, e, u)
    n = 0
    while r.scalars().time < p.total_time:
        r.step()
        n += 1
    assert n == done and r.scalars().time == sc.time


def test_solver_counters(gpu_lib):
    s = _scen("tiny_c2", 1)
    s.step()
    sc = s.scalars()
    assert sc.poisson_solves == 3
    assert sc.last_krylov_iters > 0 and sc.total_krylov_iters >= sc.last_krylov_iters
    assert sc.last_refinements >= 1
    assert sc.last_rel_residual <= s.params.tol


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["tiny_c1", "tiny_c2", "tiny_c3", "tiny_c4"])
def test_persistent_solve_matches_phase_solve(name, precision, gpu_lib):
    """krylov_kernel = 1 (one cooperative launch per pressure solve) against
    the phase-by-phase solver: same algorithm and tests, summation order of
    the dot products differs, so the solutions agree to the solver tolerance."""
    from nhwave_gb300 import fields as F
    from conftest import rel_l2
    a = _scen(name, precision)
    b = _scen(name, precision, krylov_kernel=1)
    for _ in range(3):
        assert a.step() == 0
        assert b.step() == 0
    lim = 1e-8 if precision == 0 else 1e-6
    for f in ("ETA", "P", "U", "W"):
        fid = getattr(F, f)
        sl = a.shape.interior(fid)
        r = rel_l2(b.get(fid)[sl], a.get(fid)[sl])
        assert r < lim, f"{name} {f}: {r:.3e}"
    assert np.array_equal(a.get(F.MASK), b.get(F.MASK))
    sa, sb = a.scalars(), b.scalars()
    assert sa.poisson_solves == sb.poisson_solves
    # FP32 inner solves stop at slightly different points when the dot
    # products are summed in another order: the counts agree to about 10 %
    assert abs(sa.total_krylov_iters - sb.total_krylov_iters) <= max(3, 0.1 * sa.total_krylov_iters)
    assert sb.last_rel_residual <= b.params.tol


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["tiny_c1", "tiny_c2", "tiny_c3", "tiny_c4"])
def test_gmres_matches_bicgstab(name, precision, gpu_lib):
    """GMRES (krylov_kernel = 2) against BiCGSTAB (the default) with the same
    multigrid preconditioner and refinement loop: both solve each step's
    pressure system to TOL, so the fields agree to the solver tolerance, and
    GMRES applies the preconditioner at most as often."""
    from nhwave_gb300 import fields as F
    from conftest import rel_l2
    a = _scen(name, precision)
    b = _scen(name, precision, krylov_kernel=2)
    for _ in range(3):
        assert a.step() == 0
        assert b.step() == 0
    lim = 1e-8 if precision == 0 else 1e-6
    for f in ("ETA", "P", "U", "W"):
        fid = getattr(F, f)
        sl = a.shape.interior(fid)
        r = rel_l2(b.get(fid)[sl], a.get(fid)[sl])
        assert r < lim, f"{name} {f}: {r:.3e}"
    assert np.array_equal(a.get(F.MASK), b.get(F.MASK))
    sa, sb = a.scalars(), b.scalars()
    assert sb.last_rel_residual <= b.params.tol
    # one GMRES iteration is one V-cycle, one BiCGSTAB iteration two
    assert sb.total_krylov_iters <= 2 * sa.total_krylov_iters


@pytest.mark.parametrize("precision", [0, 1])
def test_smoother_timing_leaves_the_run_unchanged(precision, gpu_lib):
    """nhw_time_smoother times the level-0 half-sweep on the handle's own
    operator: a positive time, and the next steps equal those of a run that
    was never timed, bit for bit (only a preconditioner scratch vector and a
    device buffer of its own are written)."""
    from nhwave_gb300 import fields as F, lib
    a, b = _scen("tiny_c2", precision), _scen("tiny_c2", precision)
    for s in (a, b):
        s.step()
    us = a.time_smoother(reps=4, flush_bytes=1 << 20)
    assert 0.0 < us < 1e4
    for s in (a, b):
        for _ in range(2):
            s.step()
    for f in FIELDS:
        fid = getattr(F, f)
        assert np.array_equal(a.get(fid), b.get(fid)), f
    assert a.scalars().total_krylov_iters == b.scalars().total_krylov_iters
    h = _scen("tiny_c2", precision, non_hydro=0)
    h.step()
    with pytest.raises(lib.NhwError) as ex:
        h.time_smoother(reps=2, flush_bytes=0)
    assert ex.value.status == lib.ERR_STATE
    for s in (a, b, h):
        s.close()


@pytest.mark.parametrize("name", ["tiny_c2", "tiny_ke"])
def test_baroclinic_flag_runs_the_same_path(name, gpu_lib):
    """BAROTROPIC = F adds baropg_z's gradient of Rho - Rho0 (src/nhwave.F:
    573, 13038-13179), which is zero for the uniform density of a run without
    salinity, temperature, sediment or bubbles: the run equals BAROTROPIC = T
    bit for bit."""
    from nhwave_gb300 import fields as F
    a = _scen(name, 0)
    b = _scen(name, 0, barotropic=0)
    for _ in range(3):
        a.step()
        b.step()
    for f in FIELDS:
        fid = getattr(F, f)
        assert np.array_equal(a.get(fid), b.get(fid)), f
