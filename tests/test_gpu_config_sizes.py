"""GPU parity at the configurations' own sizes, not only on small grids.

  C1  the solitary-wave channel at 256 x 8 x 10 for 100 steps: FP64 eta, P,
      U, V, W within 1e-10 relative L2 of the oracle and the mask bit for bit
      after every step; the FP32+IR form's error on the same run, per field
  C2  a 1024 x 8 x 20 strip of the submerged bar (its full length, the
      wavemaker and both sponges) for 10 steps, FP64 against the oracle
  C3  (i) the landslide beach at its full 512 x 512 x 10 for 500 steps,
      FP32+IR against FP64 on the GPU: the wet/dry mask identical after every
      step, eta within 1e-6; (ii) a 512 x 32 x 10 slice of the same beach and
      slide for 5 steps, FP64 against the oracle, with the slide's bathymetry
      copied from the oracle each step (CUDA's and the host's cosh/log differ
      in the last bit, which the slide's second time difference amplifies)

The oracle legs take minutes on one core, so they start together in a spawn
process pool when this module's first test asks for them, and run while the
GPU legs run.  Poisson TOL 1e-13 on both sides for the FP64 comparisons.
"""
import concurrent.futures as cf
import multiprocessing as mp

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-13
ORACLE_RUNS = {
    "c1": dict(name="c1", steps=100),
    "c2_strip": dict(name="c2", steps=10, N=8),
    "c3_slice": dict(name="c3", steps=5, N=32, pinned=True),
}
# FP32+IR against the FP64 oracle after the 100 C1 steps, per field (relative
# L2; U, V, W relative to the whole velocity field).  Measured on a GB300:
# eta 3.6e-7, P 1.6e-6, U 6.8e-7, V 1.5e-8, W 1.3e-7.
FP32IR_C1_BOUNDS = {"ETA": 1e-6, "P": 1e-5, "U": 5e-6, "V": 1e-7, "W": 1e-6}


def _run(spec):
    from oracle import oracle as O
    kw = dict(spec)
    return O.run_scenario(kw.pop("name"), kw.pop("steps"), tol=TOL, **kw)


@pytest.fixture(scope="module")
def oracle_runs(oracle_mod):
    pool = cf.ProcessPoolExecutor(max_workers=len(ORACLE_RUNS), mp_context=mp.get_context("spawn"))
    futs = {k: pool.submit(_run, v) for k, v in ORACLE_RUNS.items()}
    yield futs
    pool.shutdown(wait=True, cancel_futures=True)


def _gpu(name, precision=0, tol=TOL, **kw):
    from nhwave_gb300 import lib, scenarios as S
    p, d, e, u = S.make(name, precision=precision, seed=7, **kw)
    p.tol, p.itmax = tol, 20000
    return lib.Scenario(p, d, e, u)


def _interior(g, name, arr):
    from nhwave_gb300 import fields as F
    return arr[g.shape.interior(getattr(F, name))]


def _errors(g, ref):
    """Relative L2 of eta and P, and of U, V, W against the whole velocity field."""
    from nhwave_gb300 import fields as F
    out = {}
    for f in ("ETA", "P"):
        out[f] = rel_l2(_interior(g, f, g.get(getattr(F, f))), _interior(g, f, ref[f]))
    vref = np.sqrt(sum(np.linalg.norm(_interior(g, c, ref[c])) ** 2 for c in ("U", "V", "W")))
    for c in ("U", "V", "W"):
        out[c] = float(np.linalg.norm(_interior(g, c, g.get(getattr(F, c))) - _interior(g, c, ref[c])) / vref)
    return out


def _step_checking_masks(g, masks):
    from nhwave_gb300 import fields as F
    for n, m in enumerate(masks):
        assert g.step() == 0
        assert np.array_equal(g.get(F.MASK), m), f"mask differs after step {n + 1}"


def test_c1_full_size_fp64_100_steps(oracle_runs, gpu_lib):
    ref = oracle_runs["c1"].result()
    g = _gpu("c1")
    assert (g.params.Mglob, g.params.Nglob, g.params.Kglob) == (256, 8, 10)
    _step_checking_masks(g, ref["masks"])
    err = _errors(g, ref["fields"])
    for f, r in err.items():
        assert r < 1e-10, f"C1 {f} after 100 steps: rel L2 {r:.3e}"
    sc = g.scalars()
    assert sc.run_step == ref["run_step"] and abs(sc.time - ref["time"]) <= 1e-12 * ref["time"]
    print(f"\nC1 256x8x10 FP64, 100 steps vs oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    g.close()


def test_c1_full_size_fp32ir_100_steps(oracle_runs, gpu_lib):
    """The FP32+IR form against the FP64 oracle on the same 100 C1 steps:
    eta, P, U, V and W each within its stated bound, the mask bit for bit."""
    ref = oracle_runs["c1"].result()
    g = _gpu("c1", precision=1, tol=1e-10)
    _step_checking_masks(g, ref["masks"])
    err = _errors(g, ref["fields"])
    print(f"\nC1 256x8x10 FP32+IR, 100 steps vs FP64 oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for f, r in err.items():
        assert r < FP32IR_C1_BOUNDS[f], f"C1 FP32+IR {f} after 100 steps: rel L2 {r:.3e}"
    g.close()


def test_c2_strip_fp64_10_steps(oracle_runs, gpu_lib):
    ref = oracle_runs["c2_strip"].result()
    g = _gpu("c2", N=8)
    assert (g.params.Mglob, g.params.Nglob, g.params.Kglob) == (1024, 8, 20)
    _step_checking_masks(g, ref["masks"])
    err = _errors(g, ref["fields"])
    print(f"\nC2 strip 1024x8x20 FP64, 10 steps vs oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for f, r in err.items():
        assert r < 1e-10, f"C2 strip {f} after 10 steps: rel L2 {r:.3e}"
    g.close()


def test_c3_slice_fp64_pinned_5_steps(oracle_runs, gpu_lib):
    """512 x 32 x 10 of the landslide beach, routine by routine with the
    oracle's bathymetry copied in after each update_bathymetry."""
    from nhwave_gb300 import fields as F
    ref = oracle_runs["c3_slice"].result()
    g = _gpu("c3", N=32)
    assert (g.params.Mglob, g.params.Nglob, g.params.Kglob) == (512, 32, 10)
    for n, (m, bathy) in enumerate(zip(ref["masks"], ref["bathy"])):
        assert g.estimate_dt() == 0
        g.update_bathymetry()
        for name, arr in bathy.items():
            g.set(getattr(F, name), arr)
        g.update_mask()
        g.update_vars()
        for s in (1, 2, 3):
            g.source_terms()
            g.fluxes()
            assert g.eval_duvw(s) == 0
        assert np.array_equal(g.get(F.MASK), m), f"mask differs after step {n + 1}"
    err = _errors(g, ref["fields"])
    print(f"\nC3 slice 512x32x10 FP64 pinned, 5 steps vs oracle: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    for f, r in err.items():
        assert r < 1e-10, f"C3 slice {f} after 5 steps: rel L2 {r:.3e}"
    # the beach has dry land: the mask is not trivially all ones
    assert 0 < int((_interior(g, "MASK", ref["masks"][-1]) == 0).sum())
    g.close()


def test_c3_full_size_fp32ir_vs_fp64_500_steps(gpu_lib):
    """512 x 512 x 10, TOL 1e-8 as configured: the FP32+IR form (FP32 bulk,
    FP64 depth and eta at the wet/dry threshold) keeps the FP64 form's
    wet/dry mask bit for bit after every one of 500 steps, and eta within 1e-6."""
    from nhwave_gb300 import fields as F
    g64 = _gpu("c3", precision=0, tol=1e-8)
    g32 = _gpu("c3", precision=1, tol=1e-8)
    assert (g64.params.Mglob, g64.params.Nglob, g64.params.Kglob) == (512, 512, 10)
    sl = g64.shape.interior(F.MASK)
    m0 = g64.get(F.MASK)[sl].copy()
    changed = np.zeros_like(m0, dtype=bool)
    worst = 0.0
    for n in range(500):
        assert g64.step() == 0 and g32.step() == 0
        m64, m32 = g64.get(F.MASK), g32.get(F.MASK)
        assert np.array_equal(m64, m32), f"mask differs after step {n + 1}: {int((m64 != m32).sum())} cells"
        changed |= m64[sl] != m0
        if (n + 1) % 50 == 0:
            r = rel_l2(g32.get(F.ETA)[sl], g64.get(F.ETA)[sl])
            worst = max(worst, r)
            assert r < 1e-6, f"eta after step {n + 1}: rel L2 {r:.3e}"
    s64, s32 = g64.scalars(), g32.scalars()
    print(f"\nC3 512x512x10, 500 steps: FP32+IR vs FP64 eta rel L2 <= {worst:.2e}, "
          f"{int(changed.sum())} cells changed wet/dry state, t = {s64.time:.2f} s (FP32+IR {s32.time:.2f} s)")
    g64.close()
    g32.close()
