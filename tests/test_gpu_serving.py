"""Serving loop on the device: every request gives bit-identical results
(r, v, F and rebuild count) when served alone and when served in a mix with
staggered arrivals, short ticks and slot-pool grows while other replicas are
resident; the context refuses a capacity grow beyond its budget and stays
usable."""
import copy

import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300 import workloads as W
from simulationcode_gb300.batch import ReplicaBatch
from simulationcode_gb300.serving import Request, Server

pytestmark = pytest.mark.gpu


def _requests():
    rng = np.random.default_rng(7)
    P = _lib.FP32_SPLIT
    specs = [
        (W.lj_spec(1000, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=P, seed=21), 150),
        (W.berthier_spec(900, 2, _lib.LANGEVIN, rng, dt=0.002, precision=P, seed=22), 97),
        (W.berthier_spec(2500, 3, _lib.BROWNIAN, rng, dt=1e-4, precision=P, seed=23), 130),
        (W.lj_spec(700, 2, _lib.BROWNIAN, rng, dt=1e-4, precision=P, seed=24), 61),
        (W.berthier_spec(1800, 3, _lib.NEWTONIAN, rng, dt=0.002, precision=_lib.FP64, seed=25), 88),
        (W.lj_spec(1331, 3, _lib.LANGEVIN, rng, dt=0.005, precision=P, seed=26), 120),
        (W.berthier_spec(4000, 2, _lib.BROWNIAN, rng, dt=1e-4, precision=P, seed=27), 45),
    ]
    W.relax_on_device([s for s, _ in specs], 0, steps=300)
    return specs


class TickClock:
    """time in ticks: the serving loop's clock advances one unit per tick"""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def tick(self, srv):
        self.t += 1.0

    def sleep(self, dt):
        self.t += max(dt, 1e-6)


def _serve(reqs, tick_steps, reserve_slots=0):
    clk = TickClock()
    srv = Server(budget_bytes=8 * 10 ** 9, tick_steps=tick_steps, clock=clk, reserve_slots=reserve_slots)
    done = srv.run(reqs, sleep=clk.sleep, on_tick=clk.tick)
    peak = srv.peak_active
    srv.batch.close()
    return {c.request.tag: c for c in done}, peak


def test_request_alone_equals_in_the_mix(simlib):
    specs = _requests()
    alone = {}
    for k, (s, steps) in enumerate(specs):
        got, _ = _serve([Request(copy.copy(s), steps, 0.0, tag=k)], tick_steps=64, reserve_slots=8192)
        alone[k] = got[k]
    arrivals = [0.0, 0.0, 1.0, 2.0, 2.0, 4.0, 6.0]
    mix_reqs = [Request(copy.copy(s), steps, a, tag=k) for k, ((s, steps), a) in enumerate(zip(specs, arrivals))]
    mix, peak = _serve(mix_reqs, tick_steps=16, reserve_slots=0)
    assert peak >= 4                        # their work overlapped on the device
    for k in alone:
        a, m = alone[k], mix[k]
        assert a.ok and m.ok, (a.message, m.message)
        assert a.steps_done == m.steps_done == specs[k][1]
        for x, y in zip((a.r, a.v, a.F), (m.r, m.v, m.F)):
            assert np.array_equal(x, y), k
        assert a.rebuilds == m.rebuilds


def test_context_budget_refuses_grow(simlib):
    rng = np.random.default_rng(3)
    big = W.berthier_spec(60000, 3, _lib.BROWNIAN, rng, precision=_lib.FP32_SPLIT, seed=1)
    small = W.lj_spec(512, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=_lib.FP32_SPLIT, seed=2)
    b = ReplicaBatch(0)
    b.reserve(1024, 256, 2, 128)
    held = b.device_bytes()
    b.set_budget(held + b.replica_bytes(small) + (1 << 20))
    with pytest.raises(_lib.SimMDError) as e:
        b.add(big)
    assert e.value.status == _lib.ERR_BUDGET
    assert b.device_bytes() == held             # nothing was allocated
    rid = b.add(small)                          # the context is still usable
    b.step(20)
    r, v, F = b.state(rid)
    assert np.isfinite(r).all() and np.isfinite(F).all()
    b.close()
