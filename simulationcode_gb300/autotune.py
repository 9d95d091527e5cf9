"""Autotuner for a loaded ReplicaBatch: the force pass's tile shape (particles
per work item x threads per particle), the skin (the rebuild cadence: a
larger skin means longer lists but fewer rebuilds, per replica group), the
inner skin of the force pass's filtered lists (0: no filtering) and the
number of steps per captured CUDA graph.

Each candidate is timed on the live batch with CUDA events over a short run
after a short warm-up; the trial steps are ordinary MD steps of the batch
(they advance the simulation; results do not depend on the tuning up to the
order of the force sums).  The best configuration is applied and returned.
"""
from __future__ import annotations

import dataclasses
import itertools
import json
import os
from typing import Iterable, Optional

import numpy as np

from .batch import ReplicaBatch


@dataclasses.dataclass
class TuneResult:
    tpp: int
    skin: float
    graph_steps: int
    ms_per_step: float
    trials: list
    group_skins: dict = dataclasses.field(default_factory=dict)
    work_item: int = 0
    inner_skin: float = 0.0


def _may_overflow(batch: ReplicaBatch, skin: float, skin_seen: float, margin: float = 1.15) -> bool:
    """True if a replica's longest list, scaled from the longest seen so far
    (at skins up to ``skin_seen``) by the Verlet-sphere volume, could pass its
    max_neighbors at ``skin``"""
    for rid, spec in batch.specs.items():
        seen = batch.stats(rid).max_count
        rcs = spec.verlet_force_cutoff * float(np.max(spec.D))
        grow = ((rcs + skin) / (rcs + skin_seen)) ** spec.dims
        if seen * grow * margin > spec.max_neighbors:
            return True
    return False


def autotune(batch: ReplicaBatch, *, tpps: Iterable[int] = (1, 2, 4, 8), skins: Optional[Iterable[float]] = None,
             graph_steps: Iterable[int] = (16,), warmup: int = 32, steps: int = 96, log=None,
             group_by=None, work_items: Iterable[int] = (0, 64, 32),
             inner_skins: Iterable[float] = (0.2, 0.3, 0.4)) -> TuneResult:
    """Grid search over (skin, tpp, graph steps); ``skins`` None keeps the
    replicas' configured skin.  A skin whose predicted longest list could
    overflow max_neighbors is skipped (skins are tried in increasing order).
    ``group_by(spec)``: a second pass tunes the skin of each group of
    replicas separately (the rebuild cadence that suits 2D replicas differs
    from 3D).  Last, the inner skin of the force pass's filtered lists with
    one thread per particle (kept only when it beats every configuration
    without them)."""
    base_skin = next(iter(batch.specs.values())).skin if batch.specs else 0.3
    skins = [base_skin] if skins is None else sorted(skins)
    skin_seen = base_skin
    trials = []
    best = None
    for skin, tpp, gs in itertools.product(skins, tpps, graph_steps):
        if skin > skin_seen and _may_overflow(batch, skin, skin_seen):
            if log:
                log("autotune: skin=%.2f skipped (lists could overflow max_neighbors)" % skin)
            continue
        skin_seen = max(skin_seen, skin)
        batch.set_skin(skin)
        batch.set_tuning(tpp, True, gs)
        batch.step(warmup)
        batch.timer_start()
        batch.step(steps)
        ms = batch.timer_stop() / steps
        trials.append({"tpp": tpp, "skin": skin, "graph_steps": gs, "ms_per_step": ms})
        if log:
            log("autotune: skin=%.2f tpp=%d graph_steps=%d -> %.4f ms/step" % (skin, tpp, gs, ms))
        if best is None or ms < best[3]:
            best = (tpp, skin, gs, ms)
    tpp, skin, gs, ms = best
    batch.set_skin(skin)
    batch.set_tuning(tpp, True, gs)
    # tile shape: particles per force-pass work item at the best (skin, tpp);
    # 0 = whole 128-particle tiles (split only for batches smaller than the GPU)
    item, item_ms = 0, ms
    for wi in work_items:
        if wi == 0 or wi * tpp < 32:
            continue
        batch.set_work_item(wi)
        batch.step(warmup)
        batch.timer_start()
        batch.step(steps)
        t = batch.timer_stop() / steps
        trials.append({"tpp": tpp, "skin": skin, "graph_steps": gs, "work_item": wi, "ms_per_step": t})
        if log:
            log("autotune: work item %d particles -> %.4f ms/step" % (wi, t))
        if t < item_ms:
            item, item_ms = wi, t
    batch.set_work_item(item)
    ms = item_ms
    group_skins = {}
    if group_by is not None and len(skins) > 1:
        # second pass: the skin of each group of replicas (e.g. 2D and 3D),
        # the others kept at the best common skin
        groups = {}
        for rid, spec in batch.specs.items():
            groups.setdefault(group_by(spec), []).append(rid)
        if len(groups) > 1:
            for key, rids in sorted(groups.items()):
                gbest = (skin, ms)
                for sk in skins:
                    if sk == skin:
                        continue
                    if sk > skin and _may_overflow(_Subset(batch, rids), sk, skin):
                        continue
                    for rid in rids:
                        batch.set_skin(sk, rid)
                    batch.step(warmup)
                    batch.timer_start()
                    batch.step(steps)
                    t = batch.timer_stop() / steps
                    trials.append({"tpp": tpp, "skin": skin, "group": str(key), "group_skin": sk, "graph_steps": gs,
                                   "ms_per_step": t})
                    if log:
                        log("autotune: group %s skin=%.2f -> %.4f ms/step" % (key, sk, t))
                    if t < gbest[1]:
                        gbest = (sk, t)
                for rid in rids:
                    batch.set_skin(gbest[0], rid)
                group_skins[str(key)] = gbest[0]
                ms = min(ms, gbest[1])
    # inner skin of the force pass's filtered lists (one thread per particle:
    # tried also when more threads per particle won without them)
    inner = 0.0
    if 1 in tuple(tpps) and inner_skins:
        best_tpp, inner_ms = tpp, ms
        if tpp != 1:
            batch.set_tuning(1, True, gs)
        for si in inner_skins:
            batch.set_prune(si)
            batch.step(warmup)
            batch.timer_start()
            batch.step(steps)
            t = batch.timer_stop() / steps
            trials.append({"tpp": 1, "skin": skin, "inner_skin": si, "graph_steps": gs, "ms_per_step": t})
            if log:
                log("autotune: tpp=1 inner skin %.2f -> %.4f ms/step" % (si, t))
            if t < inner_ms:
                inner, inner_ms, best_tpp = si, t, 1
        batch.set_prune(inner)
        if best_tpp != 1:
            batch.set_tuning(best_tpp, True, gs)
        tpp, ms = best_tpp, inner_ms
    return TuneResult(tpp=tpp, skin=skin, graph_steps=gs, ms_per_step=ms, trials=trials, group_skins=group_skins,
                      work_item=item, inner_skin=inner)


class _Subset:
    """the replicas ``rids`` of a batch, for the overflow prediction"""

    def __init__(self, batch, rids):
        self._b = batch
        self.specs = {r: batch.specs[r] for r in rids}

    def stats(self, rid):
        return self._b.stats(rid)


TUNED_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json")


def group_key(spec) -> str:
    """the replica group of the per-group skin: '2D' or '3D'"""
    return "%dD" % spec.dims


def load_tuned(workload: str, path: str = TUNED_PATH) -> Optional[dict]:
    """the stored tuning of a workload ({"tpp", "graph_steps", "skins"}) or
    None"""
    try:
        with open(path) as f:
            return json.load(f).get(workload)
    except (OSError, ValueError):
        return None


def skin_for(tuned: Optional[dict], spec) -> float:
    """the skin a stored tuning gives a replica (its configured skin if none)"""
    if tuned is None:
        return spec.skin
    return float(tuned.get("skins", {}).get(group_key(spec), spec.skin))


def apply_tuned(batch: ReplicaBatch, tuned: dict, graphs: bool = True):
    """set a batch to a stored tuning: per-group skins, threads per particle,
    steps per captured graph, tile shape and the inner skin of the filtered
    lists (turned off before a threads-per-particle change, since filtered
    lists need one thread per particle)"""
    for rid, spec in list(batch.specs.items()):
        sk = skin_for(tuned, spec)
        if sk != spec.skin:
            batch.set_skin(sk, rid)
    tpp, inner = int(tuned.get("tpp", 1)), float(tuned.get("inner_skin", 0.0))
    if batch.inner_skin > 0 and (tpp != 1 or inner == 0):
        batch.set_prune(0.0)
    batch.set_tuning(tpp, graphs, int(tuned.get("graph_steps", 16)))
    batch.set_work_item(int(tuned.get("work_item", 0)))
    if inner > 0:
        batch.set_prune(inner)


def as_tuned(result: TuneResult, batch: ReplicaBatch) -> dict:
    """a TuneResult in the stored form"""
    skins = {}
    for spec in batch.specs.values():
        skins[group_key(spec)] = float(spec.skin)
    return {"tpp": result.tpp, "graph_steps": result.graph_steps, "skins": skins, "work_item": result.work_item,
            "inner_skin": result.inner_skin}

