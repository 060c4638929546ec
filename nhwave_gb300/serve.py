"""Continuous-batching request loop: many scenarios served from one GPU.

Each request is one scenario (an ``nhw_params`` image plus its bathymetry and
initial state) to integrate until its own TOTAL_TIME / SIM_STEPS.  The loop

* admits queued requests first-come first-served while their device memory
  (``nhw_device_bytes``, found before allocating) fits the HBM budget;
* keeps every admitted scenario's state resident on the device;
* advances all admitted scenarios together: a round is ``steps_per_round``
  ensemble steps, one CUDA graph launch each (``nhw_ensemble_*``); members
  whose run ends inside a round are held back on the device by their own
  gate, so each result is exactly its scenario's own end state;
* between rounds retires finished requests (their result fields are copied
  out, their memory freed) and admits newly arrived ones -- requests that
  arrive while others are on the GPU join the batch as memory frees up;
* can preempt a running request (``preempt``): its state is checkpointed to
  host memory and its device memory freed, and it resumes bit for bit when
  it is admitted again.

Time-to-solution of a request = the wall time from its arrival to the end of
the round in which it finished.  ``stats()`` reports p50/p99 and throughput in
cell-updates/s.  A scenario's results do not depend on which other scenarios
share its rounds (its kernels and its solver are its own).

The reference has no request loop (one scenario per program run); this is the
serving layer around the time-step path.
"""
from __future__ import annotations

import collections
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
        self.used = 0
        self.next_id = 0
        self._ens: lib.Ensemble | None = None
        self._ens_key: tuple = ()
        self.cell_updates = 0
        self.rounds = 0
        self.rebuilds = 0
        self.busy_s = 0.0

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

    # ---------------------------------------------------------------- rounds
    def _admit(self):
        now = self.clock()
        while self.pending and len(self.active) < self.max_members:
            r = self.pending[0]
            if self.used + r.bytes > self.budget:
                break
            self.pending.popleft()
            r.scenario = lib.Scenario(r.params, r.depth, r.eta0, r.uvw0)
            if r.saved is not None:          # a preempted request resumes where it stopped
                r.scenario.load_state(r.saved)
                r.saved = None
            if r.admitted is None:
                r.admitted = now
            self.used += r.bytes
            self.active.append(r)

    def _ensemble(self) -> lib.Ensemble | None:
        key = tuple(r.id for r in self.active)
        if key != self._ens_key:
            if self._ens is not None:
                self._ens.close()
                self._ens = None
            if key:
                self._ens = lib.Ensemble([r.scenario for r in self.active], **self.ensemble_opts)
                self.rebuilds += 1
            self._ens_key = key
        return self._ens

    @staticmethod
    def _over(r: Request, sc) -> bool:
        return not (sc.time < r.params.total_time and sc.run_step < r.params.sim_steps)

    def round(self) -> list[int]:
        """Admit, advance every admitted scenario steps_per_round steps, retire.
        Returns the ids of the requests that finished in this round."""
        self._admit()
        ens = self._ensemble()
        if ens is None:
            return []
        t0 = self.clock()
        before = [r.scenario.scalars().run_step for r in self.active]
        try:
            ens.step(self.steps_per_round)
        except lib.NhwError:
            pass   # DT_MIN or a non-finite solve: the members concerned are retired below
        t1 = self.clock()
        self.busy_s += t1 - t0
        self.rounds += 1
        done_ids = []
        keep = []
        for r, b in zip(self.active, before):
            sc = r.scenario.scalars()
            r.steps = sc.run_step
            self.cell_updates += r.cells * (sc.run_step - b)
            failed = sc.status == lib.ERR_DT_MIN or not np.isfinite(sc.last_rel_residual)
            if self._over(r, sc) or failed:
                r.done = t1
                r.status = sc.status if sc.status else (lib.ERR_NAN if failed else lib.OK)
                for name in self.keep:
                    r.result[name] = r.scenario.get(getattr(F, name)).copy()
                r.result["time"] = sc.time
                r.result["run_step"] = sc.run_step
                done_ids.append(r.id)
                self.finished.append(r)
            else:
                keep.append(r)
        if done_ids:
            if self._ens is not None:
                self._ens.close()
                self._ens = None
                self._ens_key = ()
            for r in self.active:
                if r.id in done_ids:
                    r.scenario.close()
                    r.scenario = None
                    self.used -= r.bytes
            self.active = keep
        return done_ids

    def preempt(self, rid: int) -> bool:
        """Take an admitted request off the GPU between rounds: its complete
        state goes to host memory (nhw_save_state), its device memory is freed
        and it returns to the front of the queue; when it is admitted again it
        resumes bit for bit (nhw_load_state).  Returns False if `rid` is not
        on the GPU."""
        for r in self.active:
            if r.id == rid:
                r.saved = r.scenario.save_state()
                r.preemptions += 1
                if self._ens is not None:
                    self._ens.close()
                    self._ens = None
                    self._ens_key = ()
                r.scenario.close()
                r.scenario = None
                self.used -= r.bytes
                self.active.remove(r)
                self.pending.appendleft(r)
                return True
        return False

    def drain(self):
        """Rounds until nothing is queued or active."""
        while self.pending or self.active:
            if not self.active and self.pending and self.used + self.pending[0].bytes > self.budget:
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
        }
        if tts.size:
            out["p50_s"] = float(np.percentile(tts, 50))
            out["p99_s"] = float(np.percentile(tts, 99))
        if wall_s:
            out["wall_s"] = wall_s
            out["cell_updates_per_s"] = self.cell_updates / wall_s
        return out

    def close(self):
        if self._ens is not None:
            self._ens.close()
            self._ens = None
        for r in self.active:
            if r.scenario is not None:
                r.scenario.close()
                r.scenario = None
        self.active = []
