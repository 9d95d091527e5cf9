"""Seeded workload generators: C4 sizes and mix, C5 request shapes (ranges,
coverage of every dims / potential / dynamics combination) and that a
request's configuration matches its drawn shape."""
import math

import numpy as np

from simulationcode_gb300 import _lib
from simulationcode_gb300 import workloads as W


def test_c4_sizes_and_mix():
    sizes = W.c4_sizes()
    assert len(sizes) == 512 and sizes.min() >= 500 and sizes.max() < 16384
    assert abs(np.log(sizes).mean() - 0.5 * (math.log(500) + math.log(16384))) < 0.2


def test_c5_draws_cover_the_mix():
    d = W.c5_draws(2000, seed=9)
    N = np.array([x[0] for x in d])
    steps = np.array([x[4] for x in d])
    assert N.min() >= 256 and N.max() < 65536
    assert steps.min() >= 1000 and steps.max() < 100000
    combos = {(x[1], x[2], x[3]) for x in d}
    assert combos == {(dims, pot, dyn) for dims in (2, 3) for pot in (0, 1) for dyn in (0, 1, 2)}
    # log-uniform: the median sits near the geometric mean of the range
    assert abs(math.log(np.median(N)) - 0.5 * (math.log(256) + math.log(65536))) < 0.3


def test_c5_request_matches_its_draw():
    d = W.c5_draws(12, seed=4)
    reqs = W.c5_requests(12, seed=4)
    for (N, dims, pot, dyn, steps), (spec, st) in zip(d, reqs):
        assert (spec.N, spec.dims, spec.potential, spec.dynamics, st) == (N, dims, pot, dyn, steps)
        assert spec.precision == _lib.FP32_SPLIT and spec.kBT == 0.1
        assert spec.r.shape == (N, dims) and np.all((spec.r >= 0) & (spec.r < spec.box_size))
        if pot == _lib.POT_LJ and dyn == _lib.BROWNIAN:
            assert spec.dt == 1e-4


def test_lattice_positions_distinct_sites():
    rng = np.random.default_rng(0)
    r = W.lattice_positions(300, 3, 6.7, rng, jitter=0.0)
    assert len({tuple(x) for x in np.round(r, 9)}) == 300
