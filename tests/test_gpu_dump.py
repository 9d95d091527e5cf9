"""Asynchronous dump feed (save_data, src/Dump.jl:60-88): a dump queued at
step k and collected after later steps equals a synchronous download at step
k bit for bit, and leaves the trajectory unchanged."""
import copy

import numpy as np
import pytest

from simulationcode_gb300 import _lib
from simulationcode_gb300 import workloads as W
from simulationcode_gb300.batch import ReplicaBatch

pytestmark = pytest.mark.gpu


def _specs():
    rng = np.random.default_rng(12)
    specs = [W.lj_spec(1000, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=_lib.FP64, seed=3),
             W.berthier_spec(1500, 2, _lib.BROWNIAN, rng, dt=1e-4, precision=_lib.FP32_SPLIT, seed=4),
             W.berthier_spec(2000, 3, _lib.LANGEVIN, rng, dt=0.002, precision=_lib.FP32_SPLIT, seed=5)]
    W.relax_on_device(specs, 0)
    return specs


def _batch(specs):
    b = ReplicaBatch(0)
    ids = [b.add(copy.copy(s)) for s in specs]
    b.rebuild()
    return b, ids


def test_dump_equals_synchronous_download(simlib):
    specs = _specs()
    a, ia = _batch(specs)
    a.step(30)
    ref = [a.state(i) for i in ia]
    a.step(50)
    ref_end = [a.state(i) for i in ia]
    a.close()

    b, ib = _batch(specs)
    b.step(30)
    for k, (i, s) in enumerate(zip(ib, specs)):
        r = np.zeros((s.N, s.dims))
        v = np.zeros((s.N, s.dims))
        F = np.zeros((s.N, s.dims))
        for x in (r, v, F):
            b.host_register(x)
        b.dump_async(i, r, v, F)
        if k == 0:
            b.step(50)          # later steps run while the copy is in flight
        b.dump_wait()
        for x in (r, v, F):
            b.host_unregister(x)
        got = (r, v, F)
        want = ref[k] if k == 0 else None
        if k == 0:
            for x, y in zip(got, want):
                assert np.array_equal(x, y)
        else:
            # dumps after the 50 extra steps equal the downloads at step 80
            for x, y in zip(got, ref_end[k]):
                assert np.array_equal(x, y)
    for i, e in zip(ib, ref_end):
        for x, y in zip(b.state(i), e):
            assert np.array_equal(x, y)
    b.close()
