"""Autotuner for a loaded ReplicaBatch: threads per particle in the force pass
(tile shape TILE x T), the skin (the rebuild cadence: a larger skin means
longer lists but fewer rebuilds) and the number of steps per captured CUDA
graph.

Each candidate is timed on the live batch with CUDA events over a short run
after a short warm-up; the trial steps are ordinary MD steps of the batch
(they advance the simulation; results do not depend on the tuning up to the
order of the force sums).  The best configuration is applied and returned.
"""
from __future__ import annotations

import dataclasses
import itertools
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
             graph_steps: Iterable[int] = (16,), warmup: int = 32, steps: int = 96, log=None) -> TuneResult:
    """Grid search; ``skins`` None keeps the replicas' configured skin.  A
    skin whose predicted longest list could overflow max_neighbors is
    skipped (skins are tried in increasing order)."""
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
    return TuneResult(tpp=tpp, skin=skin, graph_steps=gs, ms_per_step=ms, trials=trials)
