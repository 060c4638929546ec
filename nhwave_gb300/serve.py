"""Continuous-batching request loop: many scenarios served from one GPU.

Each request is one scenario (an ``nhw_params`` image plus its bathymetry and
initial state) to integrate until its own TOTAL_TIME / SIM_STEPS.  The loop

* admits queued requests first-come first-served while their device memory
  (``nhw_device_bytes``, found before allocating) fits the HBM budget;
* keeps every admitted scenario's state resident on the device;
* advances all admitted scenarios together.  The requests admitted at one
  round boundary form a cohort with one ensemble graph of their own
  (``nhw_ensemble_*``), captured once when the cohort forms; a round steps
  every cohort ``steps_per_round`` ensemble steps, each cohort from a host
  thread of its own, so the cohorts' graphs run side by side on the GPU.
  Members whose run ends inside a round are held back on the device by their
  own gate, so each result is exactly its scenario's own end state;
* between rounds retires finished requests (their result fields are copied
  out) and admits newly arrived ones as a new cohort -- requests that arrive
  while others are on the GPU join as memory frees up.  A finished request's
  memory is freed with its cohort once every member of the cohort is done;
  if a queued request needs that memory sooner, the cohorts holding finished
  members are re-formed without them first.  So membership changes never
  re-capture the graphs of requests already running;
* can preempt a running request (``preempt``): its state is checkpointed to
  host memory and its device memory freed, and it resumes bit for bit when
  it is admitted again.

Time-to-solution of a request = the wall time from its arrival to the end of
the round in which it finished.  ``stats()`` reports p50/p99 and throughput in
cell-updates/s, and the wall time spent outside the stepping: forming cohorts
(graph capture, ``capture_s``), setting scenarios up (``admit_s``) and copying
results out and freeing memory (``retire_s``).  A scenario's results do not
depend on which other scenarios share its rounds (its kernels and its solver
are its own).

The reference has no request loop (one scenario per program run); this is the
serving layer around the time-step path.
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import dataclasses
import time

import numpy as np

from . import fields as F
from . import lib
from .params import NhwParams


@dataclasses.dataclass
class Request:
    id: int
    params: NhwParams
    depth: np.ndarray
    eta0: np.ndarray | None
    uvw0: np.ndarray | None
    arrival: float
    bytes: int = 0
    admitted: float | None = None
    done: float | None = None
    status: int = lib.OK
    steps: int = 0
    scenario: "lib.Scenario | None" = None
    saved: "np.ndarray | None" = None      # checkpoint while preempted
    preemptions: int = 0
    result: dict = dataclasses.field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.params.Mglob * self.params.Nglob * self.params.Kglob


@dataclasses.dataclass
class Cohort:
    """Requests admitted together, advanced by one ensemble graph."""
    members: list
    ens: "lib.Ensemble | None" = None

    def live(self):
        return [r for r in self.members if r.done is None]


class Server:
    """Request loop over the C interface (see the module docstring)."""

    def __init__(self, hbm_budget_bytes: int, precision: int | None = None, steps_per_round: int = 8,
                 max_members: int = 256, ensemble_opts: dict | None = None, keep_fields=("ETA",),
                 clock=time.perf_counter):
        self.budget = int(hbm_budget_bytes)
        self.precision = precision
        self.steps_per_round = int(steps_per_round)
        self.max_members = int(max_members)
        self.ensemble_opts = dict(ensemble_opts or {})
        self.keep = tuple(keep_fields)
        self.clock = clock
        self.pending: collections.deque[Request] = collections.deque()
        self.active: list[Request] = []
        self.finished: list[Request] = []
        self.rejected: list[Request] = []
        self.cohorts: list[Cohort] = []
        self.used = 0
        self.next_id = 0
        self.cell_updates = 0
        self.rounds = 0
        self.rebuilds = 0          # ensemble graphs captured (cohorts formed or re-formed)
        self.busy_s = 0.0          # wall time of the rounds' stepping
        self.capture_s = 0.0       # forming cohorts: ensemble graph capture + instantiation
        self.admit_s = 0.0         # scenario set-up (allocation, upload) and checkpoint loads
        self.retire_s = 0.0        # result copies and freeing of finished requests
        self._pool: cf.ThreadPoolExecutor | None = None

    # ---------------------------------------------------------------- input
    def submit(self, params: NhwParams, depth, eta0=None, uvw0=None, arrival: float | None = None) -> int:
        p = params.copy()
        if self.precision is not None:
            p.precision = self.precision
        r = Request(self.next_id, p, np.ascontiguousarray(depth, dtype=np.float64),
                    None if eta0 is None else np.ascontiguousarray(eta0, dtype=np.float64),
                    None if uvw0 is None else np.ascontiguousarray(uvw0, dtype=np.float64),
                    self.clock() if arrival is None else arrival)
        r.bytes = lib.device_bytes(p)
        self.next_id += 1
        if r.bytes > self.budget:
            r.status = lib.ERR_CAPACITY
            r.done = r.arrival
            self.rejected.append(r)
        else:
            self.pending.append(r)
        return r.id

    # ---------------------------------------------------------------- cohorts
    def _form(self, members) -> Cohort:
        t0 = self.clock()
        c = Cohort(list(members), lib.Ensemble([r.scenario for r in members], **self.ensemble_opts))
        self.capture_s += self.clock() - t0
        self.rebuilds += 1
        return c

    def _free(self, r: Request):
        r.scenario.close()
        r.scenario = None
        self.used -= r.bytes

    def _reform(self, c: Cohort, drop: Request | None = None):
        """Re-form cohort c without its finished members (and without `drop`),
        freeing their memory; returns the new cohort or None if none is left."""
        t0 = self.clock()
        c.ens.close()
        keep = []
        for r in c.members:
            if r.done is not None:
                self._free(r)
            elif r is not drop:
                keep.append(r)
        self.retire_s += self.clock() - t0
        return self._form(keep) if keep else None

    def _holding(self) -> int:
        return sum(r.bytes for c in self.cohorts for r in c.members if r.done is not None)

    def _admit(self):
        now = self.clock()
        new = []
        n_live = len(self.active)
        while self.pending and n_live + len(new) < self.max_members:
            r = self.pending[0]
            if self.used + r.bytes > self.budget:
                if self._holding() and self.used - self._holding() + r.bytes <= self.budget:
                    # finished members' memory is needed now: re-form their cohorts without them
                    self.cohorts = [c2 for c2 in (self._reform(c) if any(m.done is not None for m in c.members)
                                                  else c for c in self.cohorts) if c2 is not None]
                    continue
                break
            self.pending.popleft()
            t0 = self.clock()
            r.scenario = lib.Scenario(r.params, r.depth, r.eta0, r.uvw0)
            if r.saved is not None:          # a preempted request resumes where it stopped
                r.scenario.load_state(r.saved)
                r.saved = None
            self.admit_s += self.clock() - t0
            if r.admitted is None:
                r.admitted = now
            self.used += r.bytes
            new.append(r)
        if new:
            self.cohorts.append(self._form(new))
        self.active = [r for c in self.cohorts for r in c.live()]

    @staticmethod
    def _over(r: Request, sc) -> bool:
        return not (sc.time < r.params.total_time and sc.run_step < r.params.sim_steps)

    @staticmethod
    def _step(ens, n):
        try:
            ens.step(n)
        except lib.NhwError:
            pass   # DT_MIN or a non-finite solve: the members concerned are retired below

    def round(self) -> list[int]:
        """Admit, advance every admitted scenario steps_per_round steps, retire.
        Returns the ids of the requests that finished in this round."""
        self._admit()
        running = [c for c in self.cohorts if c.live()]
        if not running:
            return []
        t0 = self.clock()
        before = {r.id: r.scenario.scalars().run_step for c in running for r in c.live()}
        if len(running) == 1:
            self._step(running[0].ens, self.steps_per_round)
        else:
            if self._pool is None:
                self._pool = cf.ThreadPoolExecutor(max_workers=16)
            list(self._pool.map(lambda c: self._step(c.ens, self.steps_per_round), running))
        t1 = self.clock()
        self.busy_s += t1 - t0
        self.rounds += 1
        done_ids = []
        for c in running:
            for r in c.live():
                sc = r.scenario.scalars()
                r.steps = sc.run_step
                self.cell_updates += r.cells * (sc.run_step - before[r.id])
                failed = sc.status == lib.ERR_DT_MIN or not np.isfinite(sc.last_rel_residual)
                if self._over(r, sc) or failed:
                    t2 = self.clock()
                    r.done = t1
                    r.status = sc.status if sc.status else (lib.ERR_NAN if failed else lib.OK)
                    for name in self.keep:
                        r.result[name] = r.scenario.get(getattr(F, name)).copy()
                    r.result["time"] = sc.time
                    r.result["run_step"] = sc.run_step
                    done_ids.append(r.id)
                    self.finished.append(r)
                    self.retire_s += self.clock() - t2
        # a cohort whose members are all done is freed with its graph
        keep = []
        for c in self.cohorts:
            if c.live():
                keep.append(c)
            else:
                t2 = self.clock()
                c.ens.close()
                for r in c.members:
                    self._free(r)
                self.retire_s += self.clock() - t2
        self.cohorts = keep
        self.active = [r for c in self.cohorts for r in c.live()]
        return done_ids

    def preempt(self, rid: int) -> bool:
        """Take an admitted request off the GPU between rounds: its complete
        state goes to host memory (nhw_save_state), its device memory is freed
        and it returns to the front of the queue; when it is admitted again it
        resumes bit for bit (nhw_load_state).  Its cohort is re-formed without
        it.  Returns False if `rid` is not running on the GPU."""
        for i, c in enumerate(self.cohorts):
            for r in c.live():
                if r.id == rid:
                    r.saved = r.scenario.save_state()
                    r.preemptions += 1
                    c2 = self._reform(c, drop=r)
                    self._free(r)
                    self.cohorts[i:i + 1] = [c2] if c2 is not None else []
                    self.active = [q for c3 in self.cohorts for q in c3.live()]
                    self.pending.appendleft(r)
                    return True
        return False

    def drain(self):
        """Rounds until nothing is queued or active."""
        while self.pending or self.active:
            if (not self.active and self.pending
                    and self.used - self._holding() + self.pending[0].bytes > self.budget):
                raise RuntimeError("request loop stalled: a queued request never fits the budget")
            self.round()

    def serve(self, arrivals):
        """Replay an arrival stream in real time: ``arrivals`` is a list of
        (offset_seconds, params, depth, eta0, uvw0), submitted when the wall
        clock reaches start + offset; returns when every request finished."""
        arrivals = sorted(arrivals, key=lambda a: a[0])
        start = self.clock()
        i = 0
        while i < len(arrivals) or self.pending or self.active:
            now = self.clock()
            while i < len(arrivals) and start + arrivals[i][0] <= now:
                off, p, d, e, u = arrivals[i]
                self.submit(p, d, e, u, arrival=start + off)
                i += 1
            if not self.pending and not self.active:
                if i < len(arrivals):
                    time.sleep(max(0.0, start + arrivals[i][0] - self.clock()))
                continue
            self.round()
        return self.stats(wall_s=self.clock() - start)

    # ---------------------------------------------------------------- output
    def stats(self, wall_s: float | None = None) -> dict:
        tts = np.array([r.done - r.arrival for r in self.finished], dtype=np.float64)
        out = {
            "requests": len(self.finished),
            "rejected": len(self.rejected),
            "rounds": self.rounds,
            "ensemble_rebuilds": self.rebuilds,
            "cell_updates": int(self.cell_updates),
            "busy_s": self.busy_s,
            "capture_s": self.capture_s,
            "admit_s": self.admit_s,
            "retire_s": self.retire_s,
        }
        if tts.size:
            out["p50_s"] = float(np.percentile(tts, 50))
            out["p99_s"] = float(np.percentile(tts, 99))
        if wall_s:
            out["wall_s"] = wall_s
            out["cell_updates_per_s"] = self.cell_updates / wall_s
            out["capture_share"] = self.capture_s / wall_s
        return out

    def close(self):
        for c in self.cohorts:
            if c.ens is not None:
                c.ens.close()
            for r in c.members:
                if r.scenario is not None:
                    self._free(r)
        self.cohorts = []
        self.active = []
        if self._pool is not None:
            self._pool.shutdown()
            self._pool = None
