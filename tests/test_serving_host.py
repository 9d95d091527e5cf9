"""Host logic of the serving loop (admission, ticks, retirement, failures)
against a fake batch: no device, no library calls."""
import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300.batch import ReplicaSpec
from simulationcode_gb300.serving import Request, Server, poisson_arrivals


class FakeStats:
    def __init__(self):
        self.overflow = 0
        self.nonfinite = 0
        self.rebuilds = 0


class FakeBatch:
    """stands in for ReplicaBatch: each replica's "state" counts its steps"""

    def __init__(self, pool_bytes=None):
        self.reps = {}
        self.next = 0
        self.budget = 0
        self.pool_bytes = pool_bytes
        self.log = []
        self.fail_next = {}

    def set_budget(self, b):
        self.budget = b

    def reserve(self, *a):
        pass

    def replica_bytes(self, spec):
        return spec.N * 100

    def add(self, spec):
        used = sum(self.replica_bytes(s) for s, _, _ in self.reps.values())
        if self.pool_bytes is not None and used + self.replica_bytes(spec) > self.pool_bytes:
            raise _lib.SimMDError(_lib.ERR_BUDGET, "pool")
        rid = self.next
        self.next += 1
        self.reps[rid] = (spec, [0], FakeStats())
        self.log.append(("add", rid))
        return rid

    def remove(self, rid):
        del self.reps[rid]
        self.log.append(("remove", rid))

    def step_async_status(self, k):
        st = _lib.OK
        for rid, (spec, steps, stats) in self.reps.items():
            steps[0] += k
            if self.fail_next.pop(spec.seed, False):
                stats.overflow = 1
                st = _lib.ERR_NEIGHBOR_OVERFLOW
        self.log.append(("step", k, tuple(sorted(self.reps))))
        return st

    def state(self, rid):
        spec, steps, _ = self.reps[rid]
        r = np.full((spec.N, spec.dims), float(steps[0]))
        return r, r.copy(), r.copy()

    def stats(self, rid):
        return self.reps[rid][2]


def spec(N, seed=1):
    return ReplicaSpec(dims=3, potential=0, dynamics=0, N=N, box_size=10.0, force_cutoff2=6.25, skin=0.3,
                       verlet_force_cutoff=2.5, r=np.zeros((N, 3)), D=np.ones(N), seed=seed, max_neighbors=64)


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-9)


def make_server(fb, clock, budget=10 ** 9, tick=16):
    return Server(fb, budget_bytes=budget, tick_steps=tick, clock=clock)


def test_exact_steps_and_overlap():
    fb, clk = FakeBatch(), Clock()
    srv = make_server(fb, clk, tick=16)

    def on_tick(s):
        clk.t += 1.0

    reqs = [Request(spec(100 + k, seed=k), steps, arrival) for k, (steps, arrival) in
            enumerate([(40, 0.0), (7, 0.0), (100, 1.5), (33, 2.5), (16, 9.0)])]
    done = srv.run(reqs, sleep=clk.sleep, on_tick=on_tick)
    assert len(done) == 5 and all(c.ok for c in done)
    for c in done:
        assert c.steps_done == c.request.steps
        assert np.all(c.r == c.request.steps)     # the replica ran exactly its steps
    # ticks never longer than the fewest remaining steps, nor than tick_steps
    ks = [e[1] for e in fb.log if e[0] == "step"]
    assert max(ks) <= 16
    # a later request was admitted while earlier ones were running
    adds = [i for i, e in enumerate(fb.log) if e[0] == "add"]
    first_step = min(i for i, e in enumerate(fb.log) if e[0] == "step")
    assert any(a > first_step for a in adds)
    assert any(len(e[2]) >= 2 for e in fb.log if e[0] == "step")
    s = srv.summary()
    assert s["completed"] == 5 and s["p99_s"] >= s["p50_s"] >= 0


def test_budget_admission_fifo():
    fb, clk = FakeBatch(), Clock()
    budget = 250 * 100          # room for 250 particles
    srv = make_server(fb, clk, budget=budget, tick=8)
    seen = []

    def on_tick(s):
        seen.append(s.used)
        assert s.used <= budget
        clk.t += 1.0

    reqs = [Request(spec(n, seed=k), 20, 0.0) for k, n in enumerate([200, 100, 50, 240])]
    done = srv.run(reqs, sleep=clk.sleep, on_tick=on_tick)
    assert all(c.ok for c in done)
    order = [e[1] for e in fb.log if e[0] == "add"]
    assert order == sorted(order)               # admitted first come first served
    # the 100-particle request had to wait for the 200 one (250 budget)
    first = [e for e in fb.log if e[0] == "step"][0]
    assert len(first[2]) == 1


def test_request_larger_than_budget_fails_alone():
    fb, clk = FakeBatch(), Clock()
    srv = make_server(fb, clk, budget=1000 * 100)
    reqs = [Request(spec(5000, seed=1), 10, 0.0), Request(spec(100, seed=2), 10, 0.0)]
    done = srv.run(reqs, sleep=clk.sleep, on_tick=lambda s: None)
    by = {c.request.spec.seed: c for c in done}
    assert by[1].status == _lib.ERR_BUDGET and by[2].ok


def test_pool_refusal_waits():
    # the context refuses a capacity grow (simmd_set_budget): the request
    # waits until a resident replica leaves
    fb, clk = FakeBatch(pool_bytes=300 * 100), Clock()
    srv = make_server(fb, clk, budget=10 ** 9, tick=8)
    reqs = [Request(spec(200, seed=1), 24, 0.0), Request(spec(200, seed=2), 8, 0.0)]
    done = srv.run(reqs, sleep=clk.sleep, on_tick=lambda s: None)
    assert all(c.ok for c in done)
    assert [c.request.spec.seed for c in done] == [1, 2]


def test_failure_retires_only_that_replica():
    fb, clk = FakeBatch(), Clock()
    fb.fail_next[2] = True
    srv = make_server(fb, clk, tick=8)
    reqs = [Request(spec(100, seed=k), 40, 0.0) for k in (1, 2, 3)]
    done = srv.run(reqs, sleep=clk.sleep, on_tick=lambda s: None)
    by = {c.request.spec.seed: c for c in done}
    assert by[2].status == _lib.ERR_NEIGHBOR_OVERFLOW and by[2].steps_done == 8
    assert by[1].ok and by[3].ok and by[1].steps_done == 40


def test_cancel_waiting_and_running():
    fb, clk = FakeBatch(), Clock()
    srv = make_server(fb, clk, budget=150 * 100, tick=8)
    a, b = Request(spec(100, seed=1), 64, 0.0), Request(spec(100, seed=2), 64, 0.0)
    srv.submit(a)
    srv.submit(b)
    srv.admit()
    assert len(srv.active) == 1 and len(srv.waiting) == 1
    assert srv.cancel(b)
    srv.tick()
    assert srv.cancel(a)
    st = {c.request.spec.seed: c for c in srv.completions}
    assert st[1].status == _lib.ERR_NOT_FOUND and st[1].steps_done == 8
    assert st[2].status == _lib.ERR_NOT_FOUND and st[2].steps_done == 0
    assert not srv.active and not fb.reps


def test_submit_checks():
    fb, clk = FakeBatch(), Clock()
    srv = make_server(fb, clk)
    with pytest.raises(ValueError):
        srv.submit(Request(spec(10), -1))
    s = spec(10)
    s.max_neighbors = 4096
    with pytest.raises(ValueError):
        srv.submit(Request(s, 10))


def test_poisson_arrivals_rate():
    rng = np.random.default_rng(0)
    t = poisson_arrivals(20000, 8.0, rng)
    assert np.all(np.diff(t) > 0)
    assert abs(len(t) / t[-1] - 8.0) < 0.3
