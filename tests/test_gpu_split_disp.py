"""Split precision keeps the displacement since the last rebuild as the
fixed-point difference X - X_rebuild (exact integers, u = L / 2^32 per unit)
instead of an FP64 running sum:

  * the skin trigger: stepping a split-precision replica one step at a time,
    a rebuild happens exactly at the steps where the host-side maximum of
    |r - r_rebuild| (minimum image, FP64) first exceeds skin/2 (within a few
    u), and never before;
  * the displacement the device reports equals r - r_rebuild within 3u;
  * a displacement set by the host (simmd_set_state_r) is reported back
    within 3u, and host-set positions without a displacement keep it.
"""
import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300.batch import ReplicaBatch
from simulationcode_gb300 import workloads as W
from gpu_helpers import wrap_diff

pytestmark = pytest.mark.gpu


def _spec(seed=5, skin=0.12):
    rng = np.random.default_rng(seed)
    s = W.berthier_spec(600, 3, _lib.BROWNIAN, rng, dt=1e-3, precision=_lib.FP32_SPLIT, seed=seed, skin=skin)
    b = ReplicaBatch(0)
    i = b.add(s)
    b.rebuild()
    b.relax(200, 1e-3, 0.05)
    s.r = b.state(i)[0]
    b.close()
    return s


def _disp(b, rid, s):
    d = np.zeros((s.N, s.dims))
    _lib.check(b.lib.simmd_download_r(b.ctx, rid, None, None, None, _lib.ptr(d)))
    return d


def test_split_skin_trigger_follows_host_displacement(simlib):
    s = _spec()
    b = ReplicaBatch(0, graphs=False)
    rid = b.add(s)
    b.rebuild()
    L, u = s.box_size, s.box_size / 2.0 ** 32
    r_ref = b.state(rid)[0]
    rb = b.stats(rid).rebuilds
    fired = 0
    for step in range(300):
        b.step(1)
        r = b.state(rid)[0]
        m = np.sqrt((wrap_diff(r, r_ref, L) ** 2).sum(1)).max()
        rb2 = b.stats(rid).rebuilds
        if rb2 > rb:
            assert m > s.skin / 2 - 5 * u, (step, m)
            fired += 1
            r_ref = r
        else:
            assert m <= s.skin / 2 + 4 * u, (step, m)
            assert np.abs(_disp(b, rid, s) - wrap_diff(r, r_ref, L)).max() <= 3 * u
        rb = rb2
    assert fired >= 3
    b.close()


def test_split_displacement_set_by_host(simlib):
    s = _spec(seed=6, skin=0.3)
    b = ReplicaBatch(0)
    rid = b.add(s)
    b.rebuild()
    b.step(3)
    L, u = s.box_size, s.box_size / 2.0 ** 32
    d0 = np.random.default_rng(1).uniform(-0.05, 0.05, (s.N, s.dims))
    _lib.check(b.lib.simmd_set_state_r(b.ctx, rid, None, None, None, _lib.ptr(np.ascontiguousarray(d0))))
    assert np.abs(_disp(b, rid, s) - d0).max() <= 3 * u
    # positions moved by the host without a displacement: the displacement is kept
    r = b.state(rid)[0]
    r2 = np.mod(r + 0.01, L)
    _lib.check(b.lib.simmd_set_state_r(b.ctx, rid, _lib.ptr(np.ascontiguousarray(r2)), None, None, None))
    assert np.abs(_disp(b, rid, s) - d0).max() <= 4 * u
    b.close()
