"""GPU: the bounded waits of the persistent pressure solve.

The solve's grid barrier polls with a spin limit.  Here the test hook
`test_barrier_extra` makes the barrier wait for one block that does not
exist: the wait runs out (about a second), the block sets the error word,
every later barrier returns at once, every loop still ends (ITMAX is small
here), and the host reads NHW_ERR_TIMEOUT.  Nothing faults or hangs; the
same process then steps an ordinary scenario normally."""
import time

import pytest

pytestmark = pytest.mark.gpu


def test_barrier_wait_runs_out_and_reports_timeout(gpu_lib):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make("tiny_c1", precision=1, seed=3)
    p.krylov_kernel = 1
    p.test_barrier_extra = 1
    p.itmax = 20
    g = lib.Scenario(p, d, e, u)
    t0 = time.perf_counter()
    with pytest.raises(lib.NhwError) as ex:
        g.step()
    elapsed = time.perf_counter() - t0
    assert ex.value.status == lib.ERR_TIMEOUT
    assert elapsed < 60.0
    g.close()
    # the context is still usable
    p2, d2, e2, u2 = S.make("tiny_c1", precision=1, seed=3)
    h = lib.Scenario(p2, d2, e2, u2)
    assert h.step() == lib.OK
    assert h.scalars().run_step == 1
    h.close()
