"""Serving: a continuous-batching request loop over one libsimmd context.

A request is one independent replica (its own N, dims, potential, dynamics,
precision, box and seed) plus a step count.  The server keeps every admitted
replica resident on the device and advances all of them together, one
"tick" (a bounded number of steps, all replicas in the same launches) at a
time.  Between ticks it

  * retires the replicas whose step count is reached (their final r, v, F are
    downloaded and the slots go back to the pool),
  * admits waiting requests, first come first served, while the sum of the
    admitted replicas' device footprints (``simmd_replica_bytes``) stays
    within the HBM budget; the context itself is capped by
    ``simmd_set_budget``, so a capacity grow that would pass the budget is
    refused and the request waits.

A tick is never longer than the fewest steps any admitted replica still
needs, so every replica runs exactly its requested steps.  Results do not
depend on what else is in the batch or on how the steps were split into
ticks: a replica's slot layout, neighbour lists, reductions and noise depend
only on the replica (per-replica cell sort with ties by particle id,
per-replica reductions in a fixed order, Philox noise keyed by the replica's
seed, step and particle id), and capacity grows keep the lists
(tile-major layout), so an admission never triggers a rebuild of a resident
replica.  The same request therefore gives bit-identical results alone and in
any mix.

There is no counterpart in the reference (its driver runs one system per
Julia process, src/MD.jl:680-719); the per-replica physics is the same path.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time
from typing import Callable, Deque, Dict, List, Optional

import numpy as np

from . import _lib
from .batch import ReplicaSpec

DEFAULT_BUDGET = 150 * 10 ** 9


@dataclasses.dataclass
class Request:
    spec: ReplicaSpec
    steps: int
    arrival: float = 0.0          # seconds from the start of ``Server.run``
    tag: object = None


@dataclasses.dataclass
class Completion:
    request: Request
    status: int                   # 0 = ok, else a simmd status (the replica was dropped)
    message: str
    admitted: float
    finished: float
    steps_done: int
    r: Optional[np.ndarray] = None
    v: Optional[np.ndarray] = None
    F: Optional[np.ndarray] = None
    rebuilds: int = 0

    @property
    def latency(self) -> float:
        return self.finished - self.request.arrival

    @property
    def ok(self) -> bool:
        return self.status == _lib.OK


@dataclasses.dataclass
class _Active:
    request: Request
    rid: int
    nbytes: int
    admitted: float
    remaining: int


class Server:
    """Continuous batching of independent replicas on one device.

    ``batch`` is a ReplicaBatch (or an object with the same methods: add,
    remove, step_async_status, state, stats, set_budget, replica_bytes);
    ``clock`` returns seconds (wall clock by default).
    """

    def __init__(self, batch=None, *, device: int = 0, budget_bytes: int = DEFAULT_BUDGET, tick_steps: int = 256,
                 clock: Callable[[], float] = time.perf_counter, reserve_slots: int = 0, reserve_cells: int = 0,
                 reserve_replicas: int = 0, max_neighbors: int = 128, download: bool = True):
        if batch is None:
            from .batch import ReplicaBatch
            batch = ReplicaBatch(device, tpp=1, graphs=True, graph_steps=16)
        self.batch = batch
        self.budget = int(budget_bytes)
        self.tick_steps = int(tick_steps)
        self.clock = clock
        self.download = download
        self.batch.set_budget(self.budget)
        # list rows fixed up front: a later K grow would rebuild every
        # resident replica
        self.batch.reserve(max(reserve_slots, 128), max(reserve_cells, 64), max(reserve_replicas, 1), max_neighbors)
        self.max_neighbors = max_neighbors
        self.waiting: Deque[Request] = collections.deque()
        self.active: Dict[int, _Active] = {}
        self.used = 0
        self.completions: List[Completion] = []
        self.ticks = 0
        self.particle_steps = 0
        self.busy_s = 0.0
        self.peak_active = 0
        self.peak_bytes = 0
        self._t0 = clock()

    # ---- time
    def now(self) -> float:
        return self.clock() - self._t0

    # ---- queue
    def submit(self, req: Request):
        if req.steps < 0:
            raise ValueError("steps < 0")
        if req.spec.max_neighbors > self.max_neighbors:
            raise ValueError("max_neighbors above the server's list rows (%d)" % self.max_neighbors)
        self.waiting.append(req)

    def cancel(self, req: Request) -> bool:
        """drop a waiting or running request (between ticks)"""
        for k, w in enumerate(self.waiting):
            if w is req:
                del self.waiting[k]
                self._finish_failed(req, _lib.ERR_NOT_FOUND, "cancelled", self.now(), 0)
                return True
        for rid, a in list(self.active.items()):
            if a.request is req:
                self._retire(rid, _lib.ERR_NOT_FOUND, "cancelled")
                return True
        return False

    # ---- admission
    def admit(self) -> int:
        """admit waiting requests (first come first served) within the budget"""
        n = 0
        while self.waiting:
            req = self.waiting[0]
            need = self.batch.replica_bytes(req.spec)
            if need > self.budget:
                self.waiting.popleft()
                self._finish_failed(req, _lib.ERR_BUDGET, "request larger than the budget", self.now(), 0)
                continue
            if self.used + need > self.budget:
                break                       # wait for memory to free up
            try:
                rid = self.batch.add(req.spec)
            except _lib.SimMDError as e:
                if e.status == _lib.ERR_BUDGET and self.active:
                    break                   # the pool cannot grow now: wait
                self.waiting.popleft()
                self._finish_failed(req, e.status, str(e), self.now(), 0)
                continue
            self.waiting.popleft()
            self.used += need
            self.active[rid] = _Active(req, rid, need, self.now(), int(req.steps))
            n += 1
            if req.steps == 0:
                self._retire(rid, _lib.OK, "")
        self.peak_active = max(self.peak_active, len(self.active))
        self.peak_bytes = max(self.peak_bytes, self.used)
        return n

    def _finish_failed(self, req, status, msg, t_adm, steps):
        self.completions.append(Completion(req, status, msg, t_adm, self.now(), steps))

    def _retire(self, rid: int, status: int, msg: str):
        a = self.active.pop(rid)
        r = v = F = None
        rebuilds = 0
        if status == _lib.OK and self.download:
            r, v, F = self.batch.state(rid)
        try:
            rebuilds = int(self.batch.stats(rid).rebuilds)
        except Exception:
            rebuilds = 0
        self.batch.remove(rid)
        self.used -= a.nbytes
        self.completions.append(Completion(a.request, status, msg, a.admitted, self.now(),
                                           int(a.request.steps) - a.remaining, r, v, F, rebuilds))

    # ---- one tick
    def tick(self) -> int:
        """advance every admitted replica by min(tick_steps, fewest remaining)
        steps; returns the steps taken"""
        if not self.active:
            return 0
        k = min(self.tick_steps, min(a.remaining for a in self.active.values()))
        t = self.clock()
        st = self.batch.step_async_status(k)
        self.busy_s += self.clock() - t
        self.ticks += 1
        self.particle_steps += k * sum(a.request.spec.N for a in self.active.values())
        for a in self.active.values():
            a.remaining -= k
        if st != _lib.OK:
            self._drop_failed(st)
        for rid in [rid for rid, a in self.active.items() if a.remaining == 0]:
            self._retire(rid, _lib.OK, "")
        return k

    def _drop_failed(self, status: int):
        """a step reported an error: retire the replicas that raised it"""
        bad = []
        for rid in self.active:
            s = self.batch.stats(rid)
            if s.overflow:
                bad.append((rid, _lib.ERR_NEIGHBOR_OVERFLOW, "neighbour list overflow"))
            elif s.nonfinite:
                bad.append((rid, _lib.ERR_NONFINITE, "non-finite state"))
        if not bad:   # not attributable to a replica: fail them all
            bad = [(rid, status, "step failed") for rid in self.active]
        for rid, code, msg in bad:
            self._retire(rid, code, msg)

    # ---- the loop
    def run(self, requests: List[Request], *, sleep: Callable[[float], None] = time.sleep,
            on_tick: Optional[Callable[["Server"], None]] = None) -> List[Completion]:
        """serve ``requests`` (arrival times relative to the start) until all
        have completed; returns the completions in finishing order"""
        pending = collections.deque(sorted(requests, key=lambda q: q.arrival))
        self._t0 = self.clock()
        while pending or self.waiting or self.active:
            now = self.now()
            while pending and pending[0].arrival <= now:
                self.submit(pending.popleft())
            self.admit()
            if self.active:
                self.tick()
                if on_tick:
                    on_tick(self)
            elif pending:
                sleep(max(0.0, pending[0].arrival - self.now()))
            elif self.waiting:
                raise RuntimeError("a waiting request cannot be admitted into an empty server")
        return self.completions

    def summary(self, completions: Optional[List[Completion]] = None) -> dict:
        cs = self.completions if completions is None else completions
        ok = [c for c in cs if c.ok]
        lat = np.array([c.latency for c in ok]) if ok else np.zeros(1)
        span = max((c.finished for c in cs), default=0.0) - min((c.request.arrival for c in cs), default=0.0)
        return {
            "requests": len(cs), "completed": len(ok), "failed": len(cs) - len(ok),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "max_s": float(lat.max()),
            "particle_steps": int(self.particle_steps),
            "particle_steps_per_s": self.particle_steps / span if span > 0 else 0.0,
            "makespan_s": span, "busy_s": self.busy_s, "ticks": self.ticks,
            "peak_active": self.peak_active, "peak_admitted_bytes": int(self.peak_bytes),
            "budget_bytes": self.budget,
        }


def loguniform_int(rng, lo, hi):
    return int(math.floor(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def poisson_arrivals(n: int, rate: float, rng) -> np.ndarray:
    """arrival times of a Poisson stream of ``rate`` per second"""
    return np.cumsum(rng.exponential(1.0 / rate, n))
