"""Autotuner selection logic against a fake batch (no device): it picks the
fastest (tpp, skin) and tile shape (particles per work item), skips skins
whose predicted lists overflow max_neighbors, and tunes each replica group's
skin in a second pass, and the inner skin of the filtered lists."""
import numpy as np

from simulationcode_gb300.autotune import autotune
from simulationcode_gb300.batch import ReplicaSpec


class Stats:
    def __init__(self, max_count):
        self.max_count = max_count


class FakeBatch:
    """step time = sum over replicas of a cost that depends on its skin and
    the batch's threads per particle; lists grow with the skin"""

    def __init__(self, specs, best2d, best3d, max_count=40, best_tpp=2, best_inner=None):
        self.specs = dict(enumerate(specs))
        self.skin = {r: s.skin for r, s in self.specs.items()}
        self.tpp = 1
        self.best = {2: best2d, 3: best3d}
        self.base_count = max_count
        self.t = 0.0
        self.calls = []
        self.item = 0
        self.best_item = 0
        self.best_tpp = best_tpp
        self.best_inner = best_inner  # None: filtered lists never pay
        self.inner_skin = 0.0

    def set_prune(self, inner_skin, rid=-1):
        assert self.tpp == 1 or inner_skin == 0
        self.inner_skin = inner_skin

    def set_skin(self, skin, rid=-1):
        for r in self.specs:
            if rid in (-1, r):
                self.skin[r] = skin
                self.specs[r].skin = skin

    def set_tuning(self, tpp, graphs=True, graph_steps=16):
        self.tpp = tpp

    def set_work_item(self, particles):
        self.item = particles

    def _ms(self):
        ms = 0.0
        for r, s in self.specs.items():
            ms += 1.0 + 5.0 * (self.skin[r] - self.best[s.dims]) ** 2
        ms *= (1.0 + 0.1 * abs(np.log2(self.tpp) - np.log2(self.best_tpp)))
        ms *= 1.0 if self.item == self.best_item else 1.05
        if self.inner_skin > 0:
            ms *= 0.9 if self.inner_skin == self.best_inner else 1.03
        return ms

    def step(self, n):
        self.t += n * self._ms()

    def timer_start(self):
        self.t = 0.0

    def timer_stop(self):
        return self.t

    def stats(self, rid):
        s = self.specs[rid]
        rcs = s.verlet_force_cutoff * float(np.max(s.D))
        return Stats(int(self.base_count * ((rcs + self.skin[rid]) / (rcs + 0.3)) ** s.dims))


def spec(dims, K=96):
    N = 64
    return ReplicaSpec(dims=dims, potential=1, dynamics=2, N=N, box_size=10.0, force_cutoff2=1.5625, skin=0.3,
                       verlet_force_cutoff=1.25, r=np.zeros((N, dims)), D=np.full(N, 1.2), max_neighbors=K)


def test_picks_fastest_and_tunes_groups():
    b = FakeBatch([spec(2), spec(3), spec(2), spec(3)], best2d=0.7, best3d=0.5)
    res = autotune(b, tpps=(1, 2, 4), skins=[0.3, 0.4, 0.5, 0.6, 0.7], warmup=1, steps=2,
                   group_by=lambda s: "%dD" % s.dims)
    assert res.tpp == 2
    assert res.skin == 0.6                       # best common skin for the mix
    assert res.group_skins == {"2D": 0.7, "3D": 0.5}
    assert [b.skin[r] for r in range(4)] == [0.7, 0.5, 0.7, 0.5]
    assert res.work_item == 0 and b.item == 0    # whole tiles are the fastest here


def test_picks_tile_shape():
    b = FakeBatch([spec(2), spec(3)], best2d=0.5, best3d=0.5)
    b.best_item = 64
    res = autotune(b, tpps=(1, 2), skins=[0.5], warmup=1, steps=2)
    assert res.work_item == 64 and b.item == 64
    assert any(t.get("work_item") == 32 for t in res.trials)


def test_overflowing_skins_are_skipped():
    # 3D lists at skin 0.3 already near max_neighbors: larger skins would overflow
    b = FakeBatch([spec(3, K=48), spec(3, K=48)], best2d=0.7, best3d=0.7, max_count=40)
    seen = []
    res = autotune(b, tpps=(1,), skins=[0.3, 0.5, 0.7], warmup=1, steps=2, log=seen.append)
    assert res.skin == 0.3
    assert any("skipped" in m for m in seen)
    assert all(t["skin"] == 0.3 for t in res.trials)


def test_inner_skin_axis_with_one_thread_per_particle():
    """with one thread per particle the inner skin of the filtered lists is
    tuned and kept only when it beats no filtering"""
    from simulationcode_gb300.autotune import as_tuned
    b = FakeBatch([spec(3), spec(2)], best2d=0.3, best3d=0.3, best_tpp=1, best_inner=0.3)
    res = autotune(b, tpps=(1, 2), skins=[0.3], warmup=1, steps=2, work_items=(0,), inner_skins=(0.2, 0.3, 0.4))
    assert res.tpp == 1 and res.inner_skin == 0.3 and b.inner_skin == 0.3
    assert as_tuned(res, b)["inner_skin"] == 0.3
    b2 = FakeBatch([spec(3), spec(2)], best2d=0.3, best3d=0.3, best_tpp=1, best_inner=None)
    res2 = autotune(b2, tpps=(1, 2), skins=[0.3], warmup=1, steps=2, work_items=(0,), inner_skins=(0.2, 0.3))
    assert res2.inner_skin == 0.0 and b2.inner_skin == 0.0
    # more threads per particle won without filtered lists: one thread per
    # particle with them is tried and kept only if faster
    b3 = FakeBatch([spec(3)], best2d=0.3, best3d=0.3, best_tpp=2, best_inner=0.3)
    res3 = autotune(b3, tpps=(1, 2), skins=[0.3], warmup=1, steps=2, work_items=(0,))
    assert res3.tpp == 1 and res3.inner_skin == 0.3 and b3.tpp == 1   # 1.1 * 0.9 < 1.0
    b4 = FakeBatch([spec(3)], best2d=0.3, best3d=0.3, best_tpp=4, best_inner=0.3)
    res4 = autotune(b4, tpps=(1, 2, 4), skins=[0.3], warmup=1, steps=2, work_items=(0,))
    assert res4.tpp == 4 and res4.inner_skin == 0.0 and b4.tpp == 4 and b4.inner_skin == 0.0


def test_apply_tuned_sets_the_inner_skin_after_threads_per_particle():
    """a stored tuning with an inner skin turns the filtered lists on after
    one thread per particle is set; one without turns them off first"""
    from simulationcode_gb300.autotune import apply_tuned
    b = FakeBatch([spec(3)], best2d=0.3, best3d=0.3, best_tpp=1, best_inner=0.3)
    apply_tuned(b, {"tpp": 1, "graph_steps": 16, "skins": {"3D": 0.5}, "inner_skin": 0.3})
    assert b.tpp == 1 and b.inner_skin == 0.3 and b.skin[0] == 0.5
    apply_tuned(b, {"tpp": 2, "graph_steps": 16, "skins": {"3D": 0.5}})
    assert b.tpp == 2 and b.inner_skin == 0.0
