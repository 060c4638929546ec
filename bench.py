"""Benchmark of the NHWAVE time-step path on GB300 (one JSON line on stdout).

Workload: the submerged-bar configuration -- 1024 x 64 x 20 cells, dx=0.025 m,
dy=0.05 m, internal INT_LIN wavemaker (T=2.02 s, a=0.01 m), 2 m sponges,
SSP-RK3, non-hydrostatic Poisson solve to TOL=1e-8 -- with seeded synthetic
bathymetry (scenarios.submerged_bar).  A step is one full NHWAVE time step
(estimate_dt, update_mask, update_vars, three RK stages each with fluxes, the
explicit update, the Poisson assembly and solve, the projection, Omega and the
sponge).  The metric is cell-updates/s = M*N*K*steps / device time.

  value   FP32+IR form, device-timed with CUDA events on the library's stream,
          state resident in HBM
  e2e     the same, end to end through the C-ABI with host buffers: upload of
          the prognostic state from pinned host memory, the steps, a download
          of eta after every step and of the 3-D state at the end
  fp64    the plain FP64 drop-in on the same workload and steps; the FP32+IR
          eta is compared with it (relative L2)

  ensemble  config 4: 256 scenarios of uneven size (the C4 generator) advanced
          together, one CUDA graph launch per ensemble step; device-timed
          over a few steps (the full 500-step run is out of a bench's reach)
  c3_landslide  config 3: the rigid landslide on the wet/dry beach at
          512 x 512 x 10, FP32+IR and FP64 device-timed over the same steps,
          the wet/dry masks compared and the fields' errors
  serving   config 5: Poisson arrivals at 50 requests/s replayed in real time
          through the continuous-batching loop under a 150 GB HBM budget;
          p50/p99 time-to-solution and cell-updates/s, FP32+IR and FP64; each
          request runs a bounded number of steps instead of 60 s of
          simulated time (stated in the line)

``--impl reference`` times the CPU restatement of the reference (the oracle;
the Fortran reference cannot be compiled on this machine) on the host cores.
Multi-GPU (``--gpus N`` under torchrun): independent replicas, one per GPU.
``--horizon c2|c3`` runs FP32+IR against FP64 over a whole simulated run
instead (masks after every step, the five fields' errors along the run).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "cell-updates/s FP32+IR vs FP64 at 1e-6 rel err in eta; ensemble p50/p99 latency"
UNIT = "cell-updates/s"
WORKLOAD = "submerged bar 1024x64x20 (dx=0.025, dy=0.05), INT_LIN wavemaker, sponges, SSP-RK3, NON_HYDRO, TOL=1e-8"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------ CPU baselines
def _oracle_sample(args):
    """Run the oracle on a strip of the workload; returns (cell updates, seconds)."""
    n_strip, steps, seed = args
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("c2", N=n_strip, seed=seed)
    o = O.Oracle(p, d, e, u)
    o.step()  # warm-up step (not timed)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step()
    dt = time.perf_counter() - t0
    return p.Mglob * p.Nglob * p.Kglob * steps, dt


def cpu_baseline_single(steps=1, n_strip=8):
    """Oracle, one core, on a 1024 x n_strip x 20 strip of the workload."""
    from oracle import oracle as O
    O.build()
    cells, secs = _oracle_sample((n_strip, steps, 0))
    return {"value": cells / secs, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"oracle (C++ FP64 restatement of the reference), 1 thread, "
                      f"1024x{n_strip}x20 strip of the workload, {steps} step(s) after 1 warm-up, "
                      f"{secs:.1f} s"}


def _ref_worker(idx, strip, warmup, steps, barrier, out):
    """One host core of the reference arm: its own 1024 x strip x 20 strip of
    the workload, set up once, stepped continuously; each timed step starts
    at a barrier with the other cores."""
    sys.path.insert(0, REPO)
    from oracle import oracle as O
    from nhwave_gb300 import scenarios as S
    p, d, e, u = S.make("c2", N=strip, seed=idx)
    o = O.Oracle(p, d, e, u)
    for _ in range(warmup):
        o.step()
    times = []
    for _ in range(steps):
        barrier.wait()
        t0 = time.perf_counter()
        o.step()
        times.append(time.perf_counter() - t0)
    sc = o.scalars()
    out.put((idx, p.Mglob * p.Nglob * p.Kglob, times, sc.total_krylov_iters / max(1, sc.poisson_solves)))


def run_reference_arm(args):
    """CPU restatement timed on all host cores: one oracle process per core,
    each owning a 1024 x 4 x 20 strip of the workload that it sets up once and
    steps continuously (W warm-up steps, then K timed ones).  A timed step
    starts on every core at once; its time is the slowest core's."""
    import multiprocessing as mp
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    strip = 4
    warmup = max(1, min(args.warmup, 2))
    barrier, out = ctx.Barrier(cores), ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(i, strip, warmup, args.steps, barrier, out))
             for i in range(cores)]
    for pr in procs:
        pr.start()
    import queue as _queue
    res = []
    try:
        for _ in procs:   # a worker that dies would otherwise leave the barrier and this wait hanging
            res.append(out.get(timeout=900 + 120 * (warmup + args.steps)))
    except _queue.Empty:
        for pr in procs:
            pr.terminate()
        raise RuntimeError("reference arm: a worker did not finish")
    for pr in procs:
        pr.join()
    cells = sum(r[1] for r in res)
    step_s = [max(r[2][k] for r in res) for k in range(args.steps)]
    t_all = sum(step_s)
    value = cells * args.steps / t_all
    iters = sum(r[3] for r in res) / len(res)
    sample = (f"oracle (C++ FP64 restatement; the Fortran reference has no compiler here), {cores} processes, "
              f"each stepping its own 1024x{strip}x20 strip of the workload ({warmup} warm-up steps, then the "
              f"timed ones; {iters:.1f} GMRES iterations per solve)")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": warmup, "ms_per_step": 1000.0 * t_all / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"1024x{strip * cores}x20 per step as {cores} strips",
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in open(self.path):
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


# ---------------------------------------------------------------- roofline
# Algorithmic bytes per unit of work of each kernel that can dominate a step:
# the compulsory reads and writes of the 3-D arrays (2-D fields, read once
# per column, are charged 1/K and left out), s = inner (Krylov) element size.
ALG_BYTES_PER_CELL = {
    "bicg_v": lambda s: 3 * s,       # read ph, r0; write v
    "bicg_t": lambda s: 3 * s,       # read sh, s; write t
    "bicg_p": lambda s: 5 * s,       # read r, p, v; write p, ph
    "bicg_s": lambda s: 4 * s,       # read r, v; write s, sh
    "bicg_xr": lambda s: 8 * s,      # read x, ph, sh, s, t, r0; write x, r
    "res64": lambda s: 3 * 8 + s,    # read x64, b64; write r64, rT
    "poisson_coef": lambda s: 3 * s + 16 * 8,  # read U, V, W; write 15 coefficients + rhs (FP64)
    "flux_x": lambda s: 10 * s,      # read U,V,W,DU,DV,DW; write Ex,Fx,Gx,Hx
    "flux_y": lambda s: 10 * s,
    "flux_z": lambda s: 7 * s,       # read U,V,W,Omega; write Fz,Gz,Hz
    "stage_explicit": lambda s: 20 * s,  # read 11 fluxes, DU,DV,DW; write DU,DV,DW (+R1 sum)
    "omega_x": lambda s: 3 * s, "omega_y": lambda s: 3 * s,
    # multigrid level 0, per unknown of the level: a half-sweep updates the
    # columns of one colour (half the unknowns), each reading its 7 operator
    # slots, b and x and writing x; restriction reads the 4 cross terms of the
    # colour-0 half and the colour-1 x, and writes b and x of a quarter as many
    # coarse unknowns; the correction pass reads and writes x of colour 0
    "mg_smooth_l0": lambda s: 5 * s,
    "mg_restrict_l0": lambda s: 3 * s,
    "mg_prolong_l0": lambda s: 1 * s,
    "projection": lambda s: 7 * s, "ssp_combine": lambda s: 9 * s, "get_uvw": lambda s: 6 * s,
}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            pk = json.load(fh)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_ncu_traffic():
    """Per-cell DRAM bytes per launch from the committed ncu summary, if any."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except Exception:
        return {}


def copy_ceiling(nbytes: int, device: int = 0) -> float:
    """GB/s of a plain device copy that moves `nbytes` (half read, half
    written) per launch, the size of one launch of the dominant kernel:
    CUDA events over 50 launches, rotating over buffers that together exceed
    the 129 MB L2 so that each launch reads from DRAM.  A kernel of this size
    cannot beat it; the measured peak of MEASURED_PEAKS.json is a 2 GiB copy."""
    import torch
    n = max(1, nbytes // 2 // 4)
    nbuf = max(2, int(math.ceil(2 * 300e6 / nbytes)))
    bufs = [(torch.empty(n, dtype=torch.float32, device=f"cuda:{device}"),
             torch.empty(n, dtype=torch.float32, device=f"cuda:{device}")) for _ in range(nbuf)]
    for a, b in bufs:
        a.fill_(1.0)
        b.copy_(a)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for q in range(50):
        a, b = bufs[q % nbuf]
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1000.0 / 50
    del bufs
    torch.cuda.empty_cache()
    return 2.0 * n * 4 / secs / 1e9


def roofline(prof, cells, elem_bytes, bulk_us=None):
    """The dominant kernel against the measured HBM peak.  `bulk_us`: its
    launch time from nhw_time_smoother (launches timed in bulk in a CUDA graph,
    the L2 evicted before each V-cycle's four); the per-launch event time of
    the profile pass, which carries the events' own cost, is kept beside it."""
    kern = prof["kernels"]
    total = sum(v[1] for v in kern.values())
    cand = {k: v for k, v in kern.items() if k in ALG_BYTES_PER_CELL}
    name, (launches, tot_ms) = max(cand.items(), key=lambda kv: kv[1][1])
    event_s = tot_ms / launches / 1000.0
    bulk = bulk_us is not None and name == "mg_smooth_l0"
    avg_s = bulk_us * 1e-6 if bulk else event_s
    alg = ALG_BYTES_PER_CELL[name](elem_bytes) * cells
    achieved = alg / avg_s / 1e9
    peak, peak_kind = load_peaks()
    tr = load_ncu_traffic().get(name)
    traffic = tr * cells if tr is not None else None
    shares = {k: round(v[1] / total, 4) for k, v in sorted(kern.items(), key=lambda kv: -kv[1][1])[:8]}
    return {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
            "traffic": traffic, "alg_bytes_per_launch": alg, "avg_launch_us": round(avg_s * 1e6, 2),
            "timing": ("CUDA events around a graph of 50 rounds of the V-cycle's four level-0 half-sweeps, "
                       "L2 evicted (256 MB write) before each round, writes timed alone and subtracted"
                       if bulk else "CUDA events around each launch of the profile pass"),
            "event_us_per_single_launch": round(event_s * 1e6, 2),
            "launches": launches, "kernel_time_shares": shares}


# ---------------------------------------------------------------- replicas
def replica_throughput(ms_local: float, cells: int, steps: int, world: int, device: str = "cpu"):
    """Whole-job throughput of `world` independent replicas (one per GPU, no
    data-path collective): every rank advanced `cells` cells `steps` steps;
    the elapsed time is the maximum over ranks.  Returns (max ms, cell-updates/s)."""
    t_max = ms_local
    if world > 1:
        import torch
        import torch.distributed as td
        tt = torch.tensor([ms_local], device=device, dtype=torch.float64)
        td.all_reduce(tt, op=td.ReduceOp.MAX)
        t_max = float(tt.item())
    return t_max, cells * steps * world / (t_max / 1000.0)


# --------------------------------------------------------- C4 and C5 legs
ENSEMBLE_MEMBERS = 256
SERVE_RATE, SERVE_WINDOW_S, SERVE_STEPS, SERVE_BUDGET = 50.0, 1.0, 100, 150 << 30


def run_ensemble(local, steps=10, warmup=3):
    """Config 4: 256 seeded members, FP32+IR, one ensemble graph per step."""
    from nhwave_gb300 import lib, scenarios as S
    from nhwave_gb300.params import NHW_FP32_IR
    specs = S.ensemble(ENSEMBLE_MEMBERS, seed=2024)
    ms = []
    for (p, d, e, u) in specs:
        p.precision = NHW_FP32_IR
        p.device = local
        ms.append(lib.Scenario(p, d, e, u))
    cells = sum(m.params.Mglob * m.params.Nglob * m.params.Kglob for m in ms)
    with lib.Ensemble(ms) as E:
        E.step(warmup)
        l0 = E.info().kernels_launched
        ms_dev = E.run_timed(steps)
        info = E.info()
    its = [m.scalars().total_krylov_iters / max(1, m.scalars().poisson_solves) for m in ms]
    for m in ms:
        m.close()
    return {"members": ENSEMBLE_MEMBERS, "cells": cells, "steps": steps, "warmup": warmup,
            "value": cells * steps / (ms_dev / 1000.0), "unit": UNIT, "ms_per_step": ms_dev / steps,
            "gpu_launches": int(info.kernels_launched - l0), "solver": int(info.opts.solver),
            "krylov_iters_per_solve_mean": round(float(sum(its) / len(its)), 1),
            "precision": "FP32+IR", "generator": "scenarios.ensemble(256, seed=2024)"}


def run_serving(local):
    """Config 5 (bounded): the request loop on a replayed Poisson stream, FP32+IR then FP64."""
    import numpy as np
    from nhwave_gb300 import scenarios as S, serve
    from nhwave_gb300.params import NHW_FP32_IR, NHW_FP64
    rng = np.random.default_rng(77)
    t, arr = 0.0, []
    gen = np.random.default_rng(2025)
    while True:
        t += float(rng.exponential(1.0 / SERVE_RATE))
        if t > SERVE_WINDOW_S:
            break
        p, d, e, u = S.ensemble_member(gen)
        p.sim_steps = SERVE_STEPS
        p.total_time = 1e30
        p.device = local
        arr.append((t, p, d, e, u))
    out = {"rate_per_s": SERVE_RATE, "window_s": SERVE_WINDOW_S, "requests": len(arr),
           "steps_per_request": SERVE_STEPS, "hbm_budget_bytes": SERVE_BUDGET,
           "note": f"each request runs {SERVE_STEPS} steps (not 60 s of simulated time, about 1200 steps of a "
                   f"C4 scenario) so that the run stays bounded"}
    eta = {}
    for name, prec in (("fp32ir", NHW_FP32_IR), ("fp64", NHW_FP64)):
        srv = serve.Server(SERVE_BUDGET, precision=prec, steps_per_round=10)
        st = srv.serve(arr)
        first = min(srv.finished, key=lambda r: r.id)
        eta[name] = first.result["ETA"]
        srv.close()
        out[name] = {k: st[k] for k in ("p50_s", "p99_s", "cell_updates_per_s", "wall_s", "rounds",
                                        "ensemble_rebuilds", "capture_s", "capture_share", "admit_s",
                                        "retire_s", "busy_s") if k in st}
    a, b = eta["fp32ir"], eta["fp64"]
    out["eta_rel_l2_fp32ir_vs_fp64_first_request"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return out


# ------------------------------------------------------------- C3 leg
def _end_state(g, F):
    import numpy as np
    return {"mask": g.get(F.MASK).copy(),
            **{k: g.get(f)[g.shape.interior(f)].astype(np.float64) for k, f in
               (("eta", F.ETA), ("u", F.U), ("v", F.V), ("w", F.W), ("p", F.P))}}


def _field_errors(a, b):
    """FP32+IR end state `a` against FP64 `b`: relative L2 of eta and p; u, v,
    w relative to the whole FP64 velocity field."""
    import numpy as np
    vnorm = math.sqrt(sum(float(np.linalg.norm(b[c])) ** 2 for c in ("u", "v", "w")))
    return {k: float(np.linalg.norm(a[k] - b[k]) / (vnorm if k in ("u", "v", "w") else np.linalg.norm(b[k])))
            for k in ("eta", "u", "v", "w", "p")}


def run_c3(local, steps=10, warmup=3):
    """Config 3: the rigid landslide on the wet/dry plane beach, 512 x 512 x 10,
    TOL 1e-8; FP32+IR and FP64 from the same state over the same steps, each
    device-timed, then the wet/dry masks compared and the fields' errors."""
    import numpy as np
    from nhwave_gb300 import fields as F, lib, scenarios as S
    from nhwave_gb300.params import NHW_FP32_IR, NHW_FP64
    out, ends = {"workload": "rigid landslide, plane beach 1:15, 512x512x10, dx=dy=2 m, TOL=1e-8",
                 "steps": steps, "warmup": warmup}, {}
    for name, prec in (("fp32ir", NHW_FP32_IR), ("fp64", NHW_FP64)):
        p, d, e, u = S.make("c3", precision=prec)
        p.device = local
        cells = p.Mglob * p.Nglob * p.Kglob
        g = lib.Scenario(p, d, e, u)
        g.run_timed(warmup)
        ms = g.run_timed(steps)
        sc = g.scalars()
        ends[name] = _end_state(g, F)
        out[name] = {"value": cells * steps / (ms / 1000.0), "unit": UNIT, "ms_per_step": ms / steps,
                     "krylov_iters_per_solve": round(sc.total_krylov_iters / max(1, sc.poisson_solves), 1),
                     "sim_time_s": sc.time}
        if prec == NHW_FP32_IR:
            g.profile(True)
            g.run_timed(3)
            prof = g.profile_report()
            g.profile(False)
            out[name]["roofline"] = roofline(prof, cells, 4, g.time_smoother(reps=20, flush_bytes=256 << 20))
        g.close()
    a, b = ends["fp32ir"], ends["fp64"]
    sl = (slice(2, -2), slice(2, -2))
    out["mask_equal"] = bool(np.array_equal(a["mask"], b["mask"]))
    out["dry_cells"] = int((b["mask"][sl] == 0).sum())
    out["fp32ir_rel_l2_vs_fp64"] = _field_errors(a, b)
    out["fp32ir_over_fp64"] = out["fp32ir"]["value"] / out["fp64"]["value"]
    return out


def run_horizon(args):
    """FP32+IR against FP64 over a whole simulated run (``--horizon c2``: the
    submerged bar's 20 s; ``c3``: the landslide's 200 s), both on the GPU
    from the same state: the wet/dry masks compared after every step, and the
    five fields' errors every ``--sample-every`` steps (also printed to stderr
    as they come).  ``--horizon-pair gmres64`` compares two FP64 runs instead,
    GMRES against BiCGSTAB: the spread that the Poisson stopping tolerance
    alone leaves between two solvers.  ``--horizon-tol`` overrides TOL.  One
    JSON line."""
    import numpy as np
    from nhwave_gb300 import build as B, fields as F, lib, scenarios as S
    from nhwave_gb300.params import NHW_FP32_IR, NHW_FP64
    B.build()
    gs = {}
    first = (NHW_FP64, 2) if args.horizon_pair == "gmres64" else (NHW_FP32_IR, 0)
    for name, (prec, kk) in (("fp32ir", first), ("fp64", (NHW_FP64, 0))):
        p, d, e, u = S.make(args.horizon, precision=prec)
        p.krylov_kernel = kk
        if args.horizon_tol:
            p.tol = args.horizon_tol
        gs[name] = lib.Scenario(p, d, e, u)
    total = gs["fp64"].params.total_time
    if args.max_steps:
        total = 1e30
    g32, g64 = gs["fp32ir"], gs["fp64"]
    m0 = g64.get(F.MASK).copy()
    ever_changed = np.zeros(m0.shape, dtype=bool)
    mask_diff_steps, first_diff, samples, n = 0, None, [], 0
    max_diff_cells, diff_cells = 0, 0
    t0 = time.perf_counter()
    while True:
        assert g64.step() == 0 and g32.step() == 0
        n += 1
        m64, m32 = g64.get(F.MASK), g32.get(F.MASK)
        ever_changed |= m64 != m0
        diff_cells = int((m64 != m32).sum())
        if diff_cells:
            mask_diff_steps += 1
            max_diff_cells = max(max_diff_cells, diff_cells)
            if first_diff is None:
                first_diff = {"step": n, "time_s": g64.scalars().time, "cells": diff_cells}
        t64 = g64.scalars().time
        done = t64 >= total or (args.max_steps and n >= args.max_steps)
        if n % args.sample_every == 0 or done:
            err = _field_errors(_end_state(g32, F), _end_state(g64, F))
            samples.append({"step": n, "time_s": round(t64, 4), "time_fp32ir_s": round(g32.scalars().time, 4),
                            "cells_changed_wet_dry": int(ever_changed.sum()), "mask_differing_steps": mask_diff_steps,
                            "mask_cells_differing_now": diff_cells, "mask_cells_differing_max": max_diff_cells,
                            "wall_s": round(time.perf_counter() - t0, 1),
                            **{k: float(f"{v:.3e}") for k, v in err.items()}})
            print("# " + json.dumps(samples[-1]), file=sys.stderr, flush=True)
        if done:
            break
    line = {"horizon": args.horizon, "pair": args.horizon_pair, "tol": g64.params.tol, "steps": n, "sim_time_s": t64, "wall_s": round(time.perf_counter() - t0, 1),
            "mask_equal_every_step": mask_diff_steps == 0, "mask_differing_steps": mask_diff_steps,
            "first_mask_difference": first_diff, "mask_cells_differing_max": max_diff_cells,
            "cells_changed_wet_dry": int(ever_changed.sum()),
            "samples": samples}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU arm
def run_gpu_arm(args):
    rank, world, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    from nhwave_gb300 import build as B, fields as F, lib, scenarios as S
    B.build()
    from nhwave_gb300.params import NHW_FP32_IR, NHW_FP64

    def make(prec):
        p, d, e, u = S.make("c2", precision=prec, seed=rank)
        p.device = local
        p.krylov_kernel = args.krylov_kernel
        return p, d, e, u

    # ---- FP32+IR, device-timed (value)
    p, d, e, u = make(NHW_FP32_IR)
    cells = p.Mglob * p.Nglob * p.Kglob
    g = lib.Scenario(p, d, e, u)
    g.run_timed(args.warmup)
    if world > 1:
        td.barrier()
    torch.cuda.synchronize()
    launches0 = g.profile_report()["launches"]
    with ClockSampler(local) as clk:
        ms = g.run_timed(args.steps)
    torch.cuda.synchronize()
    launches_timed = g.profile_report()["launches"] - launches0
    clocks = clk.summary()
    sc = g.scalars()
    iters_per_solve = sc.total_krylov_iters / max(1, sc.poisson_solves)
    t_max, value = replica_throughput(ms, cells, args.steps, world, device="cuda")
    ERR_FIELDS = {"eta": F.ETA, "u": F.U, "v": F.V, "w": F.W, "p": F.P}
    end32 = {k: g.get(f)[g.shape.interior(f)].astype(np.float64) for k, f in ERR_FIELDS.items()}
    # ---- profile pass: per-kernel CUDA events over the same number of steps
    g.profile(True)
    g.run_timed(max(1, min(args.steps, 5)))
    prof = g.profile_report()
    g.profile(False)
    smooth_us = g.time_smoother(reps=50, flush_bytes=256 << 20)
    g.close()
    if args.quick:
        if rank == 0:
            rl = roofline(prof, cells, 4, smooth_us)
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
                              "quick": True, "roofline": rl, "clocks": clocks,
                              "gpu_launches": launches_timed,
                              "krylov_iters_per_solve": round(iters_per_solve, 1)}), flush=True)
        return 0

    # ---- FP64 plain drop-in on the same workload and steps
    p64, d, e, u = make(NHW_FP64)
    g64 = lib.Scenario(p64, d, e, u)
    g64.run_timed(args.warmup)
    ms64 = g64.run_timed(args.steps)
    end64 = {k: g64.get(f)[g64.shape.interior(f)] for k, f in ERR_FIELDS.items()}
    iters64 = g64.scalars().total_krylov_iters / max(1, g64.scalars().poisson_solves)
    g64.close()
    value64 = cells * args.steps / (ms64 / 1000.0)
    # FP32+IR against FP64 after the same warm-up + timed steps: relative L2 of
    # eta and P; u, v, w relative to the whole FP64 velocity field
    vnorm = math.sqrt(sum(float(np.linalg.norm(end64[c])) ** 2 for c in ("u", "v", "w")))
    fp32_err = {k: float(np.linalg.norm(end32[k] - end64[k]) /
                         (vnorm if k in ("u", "v", "w") else np.linalg.norm(end64[k])))
                for k in ERR_FIELDS}
    eta_err = fp32_err["eta"]

    # ---- e2e through the C-ABI with host buffers
    p, d, e, u = make(NHW_FP32_IR)
    g = lib.Scenario(p, d, e, u)
    state_fields = [F.ETA, F.D, F.ETA0, F.D0, F.U, F.V, F.W, F.DU, F.DV, F.DW, F.P, F.OMEGA, F.MASK]
    host = {f: torch.from_numpy(np.ascontiguousarray(g.get(f))).pin_memory() for f in state_fields}
    eta_out = torch.empty(host[F.ETA].shape, dtype=torch.float64).pin_memory()
    outs3 = {f: torch.empty(host[f].shape, dtype=host[f].dtype).pin_memory() for f in (F.U, F.V, F.W, F.P)}
    g.run(args.warmup)
    torch.cuda.synchronize()
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h_step = eta_out.numel() * 8
    d2h_end = sum(t.numel() * t.element_size() for t in outs3.values())
    t0 = time.perf_counter()
    for f, t in host.items():
        g.set(f, t.numpy())
    for _ in range(args.steps):
        g.step()
        g.get(F.ETA, out=eta_out.numpy())
    for f, t in outs3.items():
        g.get(f, out=t.numpy())
    e2e_s = time.perf_counter() - t0
    g.close()
    e2e_val = cells * args.steps * world / e2e_s

    c3 = run_c3(local) if not args.no_c3 else None
    ens = run_ensemble(local) if not args.no_ensemble else None
    srv = run_serving(local) if not args.no_serving else None

    line = None
    if rank == 0:
        rl = roofline(prof, cells, 4, smooth_us)
        cc = copy_ceiling(rl["alg_bytes_per_launch"], local)
        rl["copy_same_bytes_gbs"] = round(cc, 1)
        rl["frac_of_copy_same_bytes"] = round(rl["achieved"] / cc, 4)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64-IR", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "precision": "FP32+IR",
                       "parallelism": f"replicas x{world}",
                       "l2": "no flush: per-step working set (~300 MB of state + Krylov vectors) exceeds the 129 MB L2",
                       "krylov_iters_per_solve": round(iters_per_solve, 1)},
            "fp64": {"value": value64, "unit": UNIT, "ms_per_step": ms64 / args.steps,
                     "krylov_iters_per_solve": round(iters64, 1)},
            "fp32ir_over_fp64": value / world / value64,
            "eta_rel_l2_vs_fp64": eta_err,
            "fp32ir_rel_l2_vs_fp64": {"steps": args.warmup + args.steps, **fp32_err},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
                    "d2h_bytes_per_step": int(d2h_step + d2h_end / args.steps),
                    "note": "state uploaded once from pinned host memory, eta read back every step"},
            "gpu_launches": int(launches_timed),
            "roofline": rl,
            "clocks": clocks,
        }
        if c3:
            line["c3_landslide"] = c3
        if ens:
            line["ensemble"] = ens
        if srv:
            line["serving"] = srv
    if world > 1:
        td.barrier()
    if rank == 0:
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_single()
        print(json.dumps(line), flush=True)
    if world > 1:
        td.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="FP32+IR timed region and profile pass only")
    ap.add_argument("--krylov-kernel", type=int, default=0, choices=[0, 1, 2],
                    help="pressure solver of the C2 legs: 0 BiCGSTAB phase by phase, 1 BiCGSTAB in one "
                         "persistent launch per solve, 2 GMRES phase by phase")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the config-4 ensemble leg")
    ap.add_argument("--no-serving", action="store_true", help="skip the config-5 serving leg")
    ap.add_argument("--no-c3", action="store_true", help="skip the config-3 landslide leg")
    ap.add_argument("--horizon", choices=["c2", "c3"],
                    help="instead of the bench line: FP32+IR against FP64 over the whole simulated run")
    ap.add_argument("--sample-every", type=int, default=200)
    ap.add_argument("--horizon-pair", choices=["fp32ir", "gmres64"], default="fp32ir",
                    help="FP32+IR against FP64 (default), or FP64 GMRES against FP64 BiCGSTAB")
    ap.add_argument("--horizon-tol", type=float, default=0.0, help="Poisson TOL of both runs (0: the config's)")
    ap.add_argument("--max-steps", type=int, default=0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.horizon:
        return run_horizon(args)
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
