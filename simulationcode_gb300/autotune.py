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

from .batch import ReplicaBatch


@dataclasses.dataclass
class TuneResult:
    tpp: int
    skin: float
    graph_steps: int
    ms_per_step: float
    trials: list


def autotune(batch: ReplicaBatch, *, tpps: Iterable[int] = (1, 2, 4), skins: Optional[Iterable[float]] = None,
             graph_steps: Iterable[int] = (16,), warmup: int = 32, steps: int = 96, log=None) -> TuneResult:
    """Grid search; ``skins`` None keeps the replicas' configured skin."""
    base_skin = next(iter(batch.specs.values())).skin if batch.specs else 0.3
    skins = [base_skin] if skins is None else list(skins)
    trials = []
    best = None
    for skin, tpp, gs in itertools.product(skins, tpps, graph_steps):
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
