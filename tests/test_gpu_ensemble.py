"""GPU: ensembles -- many scenarios advanced by one graph launch per step,
their pressure solves sharing persistent cooperative launches.

* a member's results are the same bits alone and in a mix, with either
  solver (the persistent groups' block counts depend only on a member's own
  size);
* ensemble steps agree with the same scenarios stepped one by one through
  nhw_step: bit for bit with the phase-by-phase solver on every member's
  branch (the same kernels in the same order), to the solver tolerance with
  the persistent groups;
* members whose run is over are skipped on the device, each at its own
  SIM_STEPS;
* the autotuner returns one of its candidate settings and the ensemble
  still steps correctly with it.
"""
import numpy as np
import pytest

from conftest import rel_l2, seed_ke

pytestmark = pytest.mark.gpu

FIELDS = ["ETA", "D", "U", "V", "W", "P", "OMEGA", "MASK"]


def _member(name, precision, seed=5, **attrs):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=precision, seed=seed)
    p.tol = 1e-10 if precision == 0 else 1e-8
    p.itmax = 5000
    for k, v in attrs.items():
        setattr(p, k, v)
    return lib.Scenario(p, d, e, u)


def _ensemble_members(precision):
    """Three members of uneven sizes from the C4 generator."""
    from nhwave_gb300 import scenarios as S
    out = []
    for i, (M, K) in enumerate(((40, 5), (64, 10), (32, 15))):
        p, d, e, u = S.ensemble_member(np.random.default_rng(100 + i), side=(M, M), Kchoices=(K,))
        p.precision = precision
        p.tol = 1e-10 if precision == 0 else 1e-8
        out.append((p, d, e, u))
    return out


def _mk(spec):
    from nhwave_gb300 import lib
    p, d, e, u = spec
    return lib.Scenario(p, d, e, u)


@pytest.mark.parametrize("solver", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_member_alone_equals_member_in_mix(precision, solver, gpu_lib):
    from nhwave_gb300 import fields as F, lib
    specs = _ensemble_members(precision)
    mix = [_mk(s) for s in specs]
    alone = _mk(specs[1])
    opts = dict(cells_per_block=4096, block_rows=8, coarse_sweeps=2, solver=solver)
    with lib.Ensemble(mix, **opts) as em, lib.Ensemble([alone], **opts) as ea:
        assert em.step(3) == 0
        assert ea.step(3) == 0
        for f in FIELDS:
            fid = getattr(F, f)
            x, y = mix[1].get(fid), alone.get(fid)
            assert np.array_equal(x, y), f"{f} differs between the mix and alone"
        assert mix[1].scalars().total_krylov_iters == alone.scalars().total_krylov_iters


@pytest.mark.parametrize("solver", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_matches_single_steps(precision, solver, gpu_lib):
    from nhwave_gb300 import fields as F, lib
    names = ["tiny_c1", "tiny_c2", "tiny_c3", "tiny_c4"]
    ens = [_member(n, precision) for n in names]
    ref = [_member(n, precision) for n in names]
    with lib.Ensemble(ens, solver=solver) as e:
        info = e.info()
        assert info.members == 4 and info.kernels_per_step > 0
        for _ in range(3):
            assert e.step(1) == 0
            for r in ref:
                assert r.step() == 0
    lim = 1e-8 if precision == 0 else 1e-6
    for n, a, b in zip(names, ens, ref):
        sa, sb = a.scalars(), b.scalars()
        assert sa.run_step == sb.run_step == 3
        assert abs(sa.time - sb.time) <= 1e-12 * sb.time
        assert np.array_equal(a.get(F.MASK), b.get(F.MASK)), n
        for f in ("ETA", "P", "U"):
            fid = getattr(F, f)
            sl = a.shape.interior(fid)
            if solver == 0:
                assert np.array_equal(a.get(fid), b.get(fid)), f"{n} {f} differs"
            else:
                r = rel_l2(a.get(fid)[sl], b.get(fid)[sl])
                assert r < lim, f"{n} {f}: {r:.3e}"


def test_members_stop_at_their_own_sim_steps(gpu_lib):
    from nhwave_gb300 import lib
    a = _member("tiny_c1", 1, sim_steps=2, total_time=1e9)
    b = _member("tiny_c4", 1, sim_steps=5, total_time=1e9)
    with lib.Ensemble([a, b]) as e:
        assert e.step(8) == 0
        launched = e.info().kernels_launched
    assert launched > 0
    assert a.scalars().run_step == 2
    assert b.scalars().run_step == 5


def test_autotuner_picks_a_candidate(gpu_lib):
    from nhwave_gb300 import lib
    specs = _ensemble_members(1)
    ms = [_mk(s) for s in specs]
    with lib.Ensemble(ms) as e:
        o = e.tune(1)
        assert o.solver in (0, 1)
        assert o.cells_per_block in (4096, 16384, 65536)
        assert o.block_rows in (8, 16)
        assert o.coarse_sweeps in (2, 4, 6)
        n0 = [m.scalars().run_step for m in ms]
        assert e.step(2) == 0
        assert [m.scalars().run_step for m in ms] == [x + 2 for x in n0]
        info = e.info()
        assert info.opts.cells_per_block == o.cells_per_block


@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_of_gmres_members_matches_single_steps(precision, gpu_lib):
    """Members on the GMRES solver (krylov_kernel = 2) inside one ensemble
    graph: each member's branch runs the kernels its own step would, so the
    fields agree bit for bit with the members stepped one by one."""
    from nhwave_gb300 import fields as F, lib
    names = ["tiny_c1", "tiny_c3", "tiny_c4"]
    ens = [_member(n, precision, krylov_kernel=2) for n in names]
    ref = [_member(n, precision, krylov_kernel=2) for n in names]
    with lib.Ensemble(ens, solver=0) as e:
        for _ in range(2):
            assert e.step(1) == 0
            for r in ref:
                assert r.step() == 0
    for n, a, b in zip(names, ens, ref):
        assert a.scalars().total_krylov_iters == b.scalars().total_krylov_iters, n
        for f in ("ETA", "P", "U", "MASK"):
            fid = getattr(F, f)
            assert np.array_equal(a.get(fid), b.get(fid)), f"{n} {f} differs"


@pytest.mark.parametrize("solver", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_of_the_added_boundaries_and_viscous_flow(precision, solver, gpu_lib):
    """Members that use the later rows -- viscous flow on a friction bed with
    friction walls, an Orlanski east side, cnoidal and focused inflow, the
    FLUX_LR current through both ends -- step in
    one ensemble as they step alone (bit for bit with solver 0)."""
    from nhwave_gb300 import fields as F, lib
    names = ["tiny_visc_fric", "tiny_open", "tiny_flume_con", "tiny_flume_foc", "tiny_flux_lr"]
    ens = [_member(n, precision) for n in names]
    ref = [_member(n, precision) for n in names]
    with lib.Ensemble(ens, solver=solver) as e:
        for _ in range(3):
            assert e.step(1) == 0
            for r in ref:
                assert r.step() == 0
    lim = 1e-8 if precision == 0 else 1e-6
    for n, a, b in zip(names, ens, ref):
        assert a.scalars().run_step == b.scalars().run_step == 3
        assert np.array_equal(a.get(F.MASK), b.get(F.MASK)), n
        for f in ("ETA", "P", "U", "W"):
            fid = getattr(F, f)
            if solver == 0:
                assert np.array_equal(a.get(fid), b.get(fid)), f"{n} {f} differs"
            else:
                sl = a.shape.interior(fid)
                den = max(np.linalg.norm(b.get(fid)[sl]), 1e-30)
                r = np.linalg.norm(a.get(fid)[sl] - b.get(fid)[sl]) / den
                assert r < lim, f"{n} {f}: {r:.3e}"


@pytest.mark.parametrize("precision", [0, 1])
def test_ensemble_of_the_turbulence_closures(precision, gpu_lib):
    """Members with the subgrid model, the 3-D and 2-D k-epsilon closures
    (from the same seeded turbulence) and the Smagorinsky and dynamic LES
    step in one ensemble bit for bit as they step alone, eddy viscosities
    and k-epsilon state included."""
    from nhwave_gb300 import fields as F, lib
    names = ["tiny_visc_sgs", "tiny_ke_rng", "tiny_ke2", "tiny_les", "tiny_lesdyn"]
    ens = [_member(n, precision) for n in names]
    ref = [_member(n, precision) for n in names]
    for a, b in zip(ens, ref):
        if a.params.ivturb in (3, 10):
            seed_ke(a, b)
    with lib.Ensemble(ens, solver=0) as e:
        for _ in range(3):
            assert e.step(1) == 0
            for r in ref:
                assert r.step() == 0
    for n, a, b in zip(names, ens, ref):
        assert a.scalars().run_step == b.scalars().run_step == 3
        fields = ["ETA", "P", "U", "W", "CMUVT", "CMUHT"] + (["TKE", "EPS"] if a.params.ivturb in (3, 10) else [])
        for f in fields:
            fid = getattr(F, f)
            assert np.array_equal(a.get(fid), b.get(fid)), f"{n} {f} differs"
