"""Inner (pruned) neighbour lists (simmd_set_prune): the force pass reads the
outer-list pairs within rc_ij + inner_skin, re-filtered after every rebuild
and whenever a particle has moved inner_skin/2 since the last filter.  The
dropped pairs are out of the force cutoff until then and add exactly zero,
so with one thread per particle every trajectory must be bit-identical to
the unfiltered one:

  * a mixed batch (2D/3D, LJ/Berthier, Newtonian/Langevin/Brownian, FP64 and
    split precision), graphs and direct launches, 240 steps: positions,
    velocities, forces and rebuild counts equal at every check; prunes well
    above rebuilds (the displacement trigger fires), inner lists shorter
    than the outer ones;
  * host-set positions (simmd_set_state_r) and the set-up relaxation between
    steps: still bit-identical;
  * the 512-replica workload's first 24 replicas with the stored tuning,
    100 steps: bit-identical.
"""
import copy

import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300.batch import ReplicaBatch
from simulationcode_gb300 import workloads as W
from test_gpu_batch import _mixed_specs, _relaxed

pytestmark = pytest.mark.gpu


def _pair(specs, graphs, inner):
    out = []
    for prune in (False, True):
        b = ReplicaBatch(0, graphs=graphs, graph_steps=8)
        ids = [b.add(copy.copy(s)) for s in specs]
        if prune and inner > 0:
            b.set_prune(inner)
        b.rebuild()
        out.append((b, ids))
    return out


def _same(a, b, ida, idb):
    for x, y in zip(ida, idb):
        for u, v in zip(a.state(x), b.state(y)):
            assert np.array_equal(u, v), x
        assert a.stats(x).rebuilds == b.stats(y).rebuilds


@pytest.mark.parametrize("graphs", [True, False])
def test_pruned_lists_give_bit_identical_trajectories(simlib, graphs):
    specs = _relaxed(_mixed_specs(seed=7))
    (a, ia), (b, ib) = _pair(specs, graphs, 0.08)
    for _ in range(6):
        a.step(40)
        b.step(40)
        _same(a, b, ia, ib)
    prunes, inner, outer = 0, 0, 0
    for y in ib:
        n, e = b.prune_stats(y)
        prunes += n
        inner += e
        outer += b.stats(y).list_entries
        assert n >= b.stats(y).rebuilds
    assert prunes > 2 * sum(b.stats(y).rebuilds for y in ib)
    assert 0 < inner < 0.9 * outer
    a.close()
    b.close()


def test_pruned_lists_after_host_positions_and_relaxation(simlib):
    specs = _relaxed(_mixed_specs(seed=8))
    (a, ia), (b, ib) = _pair(specs, True, 0.1)
    for batch in (a, b):
        batch.step(30)
    # positions moved by the host without a rebuild (lists kept), then steps
    rng = np.random.default_rng(2)
    for x, y, s in zip(ia, ib, specs):
        r = a.state(x)[0]
        r2 = np.mod(r + rng.uniform(-0.02, 0.02, r.shape), s.box_size)
        for batch, k in ((a, x), (b, y)):
            _lib.check(batch.lib.simmd_set_state_r(batch.ctx, k, _lib.ptr(np.ascontiguousarray(r2)), None, None,
                                                   None))
    for batch in (a, b):
        batch.step(20)
    _same(a, b, ia, ib)
    for batch in (a, b):
        batch.relax(5, 1e-3, 0.02)
        batch.step(25)
    _same(a, b, ia, ib)
    a.close()
    b.close()


def test_pruned_lists_on_the_replica_workload(simlib):
    from simulationcode_gb300 import autotune as AT
    specs = W.c4(indices=list(range(24)))
    W.relax_on_device(specs, 0)
    tuned = dict(AT.load_tuned("c4"), inner_skin=0.0)
    (a, ia), (b, ib) = _pair(specs, True, 0.0)
    AT.apply_tuned(a, tuned)
    AT.apply_tuned(b, dict(tuned, inner_skin=0.15))
    assert b.inner_skin == 0.15 and a.inner_skin == 0.0
    a.step(100)
    b.step(100)
    _same(a, b, ia, ib)
    n, e = b.prune_stats(ib[0])
    assert n > b.stats(ib[0]).rebuilds and e > 0
    a.close()
    b.close()
