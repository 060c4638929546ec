"""GPU: checkpoint / resume (nhw_checkpoint_bytes, nhw_save_state,
nhw_load_state) and serving-loop preemption built on it.

A run saved after n steps and resumed in a fresh handle -- created and set up
from the same inputs, as the reference's hot start rereads its inputs --
continues bit for bit like the run that never stopped; a checkpoint of
another grid is rejected; a request preempted off the GPU and resumed later
ends with the same bits as one served without interruption."""
import numpy as np
import pytest

from conftest import seed_ke

pytestmark = pytest.mark.gpu

FIELDS = ["ETA", "D", "HC", "U", "V", "W", "DU", "P", "OMEGA", "MASK", "ETAXL", "HFX0", "DELT2H"]


def _scen(name, precision, **attrs):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=precision, seed=9)
    p.tol = 1e-10 if precision == 0 else 1e-8
    p.itmax = 5000
    for k, v in attrs.items():
        setattr(p, k, v)
    s = lib.Scenario(p, d, e, u)
    if p.viscous_flow and p.ivturb in (3, 10):
        seed_ke(s)
    return s


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,krylov", [("tiny_c2", 0), ("tiny_c3", 0), ("tiny_c4", 0), ("tiny_flume_lin", 0),
                                         ("tiny_open", 0), ("tiny_visc", 0), ("tiny_c2", 2), ("tiny_flux_lr", 0),
                                         ("tiny_visc_sgs", 0), ("tiny_ke_rng", 0), ("tiny_les", 0),
                                         ("tiny_ke2", 0)])
def test_resume_continues_bit_for_bit(name, krylov, precision, gpu_lib):
    """krylov = 2: the GMRES solver, whose basis lies behind the checkpointed
    prefix and is rebuilt by every solve.  tiny_open: the Orlanski boundary's
    two earlier time levels are part of the checkpointed state; tiny_flux_lr:
    so are FLUX_LR's outflow velocities of the last two steps; tiny_visc:
    the sigma slopes the next viscous terms read are too; tiny_visc_sgs: and
    the cells' eddy viscosities of the last eval_turb; tiny_ke_rng: and the
    k-epsilon state."""
    from nhwave_gb300 import fields as F
    a = _scen(name, precision, krylov_kernel=krylov)
    for _ in range(4):
        a.step()
    buf = a.save_state()
    for _ in range(3):
        a.step()
    b = _scen(name, precision, krylov_kernel=krylov)
    b.load_state(buf)
    assert b.scalars().run_step == 4
    for _ in range(3):
        b.step()
    sa, sb = a.scalars(), b.scalars()
    assert (sa.time, sa.dt, sa.run_step) == (sb.time, sb.dt, sb.run_step)
    assert sa.total_krylov_iters == sb.total_krylov_iters
    extra = (["CMUVT", "CMUHT"] if a.params.viscous_flow else []) + \
        (["TKE", "EPS", "DTKE", "DEPS"] if a.params.viscous_flow and a.params.ivturb in (3, 10) else [])
    for f in FIELDS + extra:
        fid = getattr(F, f)
        assert np.array_equal(a.get(fid), b.get(fid)), f"{name} {f}"


def test_checkpoint_of_another_grid_rejected(gpu_lib):
    from nhwave_gb300 import lib
    a = _scen("tiny_c1", 1)
    a.step()
    buf = a.save_state()
    b = _scen("tiny_c2", 1)
    with pytest.raises(lib.NhwError) as ex:
        b.load_state(buf)
    assert ex.value.status == lib.ERR_ARG
    c = _scen("tiny_c1", 0)        # same grid, other precision
    with pytest.raises(lib.NhwError):
        c.load_state(buf)
    with pytest.raises(lib.NhwError):
        a.load_state(buf[:100])


def test_preempted_request_ends_like_an_uninterrupted_one(gpu_lib):
    from nhwave_gb300 import scenarios as S, serve
    p, d, e, u = S.ensemble_member(np.random.default_rng(31), side=(40, 40), Kchoices=(10,))
    p.precision = 1
    p.sim_steps = 10
    p.total_time = 1e9
    plain = serve.Server(hbm_budget_bytes=8 << 30, steps_per_round=2, keep_fields=("ETA", "P"))
    plain.submit(p, d, e, u)
    plain.drain()
    pre = serve.Server(hbm_budget_bytes=8 << 30, steps_per_round=2, keep_fields=("ETA", "P"))
    rid = pre.submit(p, d, e, u)
    pre.round()
    pre.round()
    assert pre.preempt(rid)
    assert not pre.active and pre.used == 0
    pre.drain()
    a, b = plain.finished[0], pre.finished[0]
    assert b.preemptions == 1
    assert a.result["run_step"] == b.result["run_step"] == 10
    for f in ("ETA", "P"):
        assert np.array_equal(a.result[f], b.result[f]), f
    plain.close()
    pre.close()
