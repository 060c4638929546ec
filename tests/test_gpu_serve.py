"""GPU: the continuous-batching request loop (nhwave_gb300.serve).

* a request's result is the same bits served alone and served in a mix of
  other requests that arrive while it runs;
* admission respects the HBM budget (device bytes known before allocating),
  and requests queue until memory frees up;
* every request ends at its own TOTAL_TIME / SIM_STEPS;
* stats() reports p50/p99 time-to-solution and throughput.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _req(seed, M, K, steps):
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.ensemble_member(np.random.default_rng(seed), side=(M, M), Kchoices=(K,))
    p.precision = 1
    p.sim_steps = steps
    p.total_time = 1e9
    return p, d, e, u


def test_result_same_alone_and_in_mix(gpu_lib):
    from nhwave_gb300 import serve
    target = _req(7, 48, 10, 9)
    others = [_req(10 + i, 32 + 8 * i, 5 + 5 * (i % 3), 4 + 3 * i) for i in range(4)]
    alone = serve.Server(hbm_budget_bytes=8 << 30, steps_per_round=4, keep_fields=("ETA", "U", "P"))
    alone.submit(*target)
    alone.drain()
    mix = serve.Server(hbm_budget_bytes=8 << 30, steps_per_round=4, keep_fields=("ETA", "U", "P"))
    mix.submit(*others[0])
    mix.round()                      # the target arrives while another request is on the GPU
    mix.submit(*others[1])
    tid = mix.submit(*target)
    mix.round()
    for o in others[2:]:
        mix.submit(*o)
    mix.drain()
    a = alone.finished[0]
    b = [r for r in mix.finished if r.id == tid][0]
    assert a.result["run_step"] == b.result["run_step"] == 9
    for f in ("ETA", "U", "P"):
        assert np.array_equal(a.result[f], b.result[f]), f
    assert len(mix.finished) == 5
    for r in mix.finished:
        assert r.result["run_step"] == r.params.sim_steps
    alone.close()
    mix.close()


def test_budget_admission_and_stats(gpu_lib):
    from nhwave_gb300 import lib, serve
    reqs = [_req(20 + i, 40, 5, 3 + i) for i in range(6)]
    one = lib.device_bytes(reqs[0][0])
    srv = serve.Server(hbm_budget_bytes=int(2.5 * one), steps_per_round=2)
    for r in reqs:
        srv.submit(*r)
    peak = 0
    while srv.pending or srv.active:
        srv.round()
        peak = max(peak, len(srv.active))
        assert srv.used <= srv.budget
    assert peak <= 2
    st = srv.stats(wall_s=1.0)
    assert st["requests"] == 6 and st["rejected"] == 0
    assert 0 < st["p50_s"] <= st["p99_s"]
    assert st["cell_updates"] == sum(r[0].Mglob * r[0].Nglob * r[0].Kglob * r[0].sim_steps for r in reqs)
    # a request larger than the whole budget is rejected at once
    big = _req(99, 40, 5, 3)
    srv2 = serve.Server(hbm_budget_bytes=one // 2)
    srv2.submit(*big)
    assert len(srv2.rejected) == 1 and srv2.rejected[0].status == lib.ERR_CAPACITY
    srv.close()


def test_poisson_arrivals_replayed(gpu_lib):
    from nhwave_gb300 import serve
    rng = np.random.default_rng(5)
    t = np.cumsum(rng.exponential(1.0 / 50.0, size=8))     # 50 requests/s
    arrivals = [(float(ti),) + _req(40 + i, 32, 5, 4) for i, ti in enumerate(t)]
    srv = serve.Server(hbm_budget_bytes=8 << 30, steps_per_round=2)
    st = srv.serve(arrivals)
    assert st["requests"] == 8
    assert st["cell_updates_per_s"] > 0 and st["p99_s"] >= st["p50_s"] > 0
    srv.close()
