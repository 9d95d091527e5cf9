"""Inherent-structure minimiser (find_inherent_structure,
src/InherentStructure.jl:5-56) on the device against the oracle: final
positions within 1e-8 (box units) and the same iteration count (+-2); in a
batch, every replica's result equals the replica minimised alone."""
import ctypes as C

import numpy as np
import pytest

from cases import make_case
from gpu_helpers import GpuSystem, wrap_diff
from simulationcode_gb300 import _lib
from simulationcode_gb300 import workloads as W
from simulationcode_gb300.batch import ReplicaBatch

pytestmark = pytest.mark.gpu

ARGS = dict(tolerance=1e-4, max_iterations=200000, max_step_size=0.001, dt=0.005)


# the reference's descent uses a fixed dt (v = F dt): stiff contacts need a
# smaller one to converge (at dt = 0.005 the oracle oscillates for these)
@pytest.mark.parametrize("pot,dims,N,dt", [(1, 3, 500, 0.005), (1, 2, 400, 1e-3), (0, 3, 216, 1e-3),
                                           (0, 2, 400, 5e-4)])
def test_inherent_structure_matches_oracle(simlib, oracle, pot, dims, N, dt):
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=21)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    args = dict(ARGS, dt=dt)
    st, it_ref = oracle.find_inherent_structure(ref, **args)
    assert st == 0
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    it = (C.c_int64 * 1)()
    assert simlib.simmd_inherent_structure(gpu.ctx, args["tolerance"], args["max_iterations"],
                                           args["max_step_size"], args["dt"], it) == 0
    rg = gpu.state()[0]
    assert np.abs(wrap_diff(rg, ref.r, p.box_size)).max() < 1e-8
    assert abs(int(it[0]) - it_ref) <= 2
    gpu.close()


def test_not_converged_status(simlib, oracle):
    p, r, v, D, rc = make_case(1, 3, 0, 500, seed=22)
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    it = (C.c_int64 * 1)()
    st = simlib.simmd_inherent_structure(gpu.ctx, 1e-12, 50, 0.001, 0.005, it)
    assert st == _lib.ERR_NOT_CONVERGED and it[0] == 50
    gpu.step(5)                    # the context keeps working afterwards
    gpu.close()


def test_batch_minimisation_equals_alone(simlib):
    rng = np.random.default_rng(4)
    specs = [W.berthier_spec(600, 2, _lib.BROWNIAN, rng, precision=_lib.FP32_SPLIT, seed=1),
             W.lj_spec(512, 3, _lib.NEWTONIAN, rng, precision=_lib.FP64, seed=2),
             W.berthier_spec(900, 3, _lib.LANGEVIN, rng, precision=_lib.FP32_SPLIT, seed=3)]
    W.relax_on_device(specs, 0, steps=100)
    args = dict(ARGS, dt=1e-3, max_iterations=3000, allow_not_converged=True)
    mix = ReplicaBatch(0)
    ids = [mix.add(s) for s in specs]
    its = mix.inherent_structure(**args)
    for rid, s in zip(ids, specs):
        alone = ReplicaBatch(0)
        a = alone.add(s)
        ita = alone.inherent_structure(**args)
        assert ita[a] == its[rid]
        assert np.array_equal(alone.state(a)[0], mix.state(rid)[0])
        alone.close()
    mix.close()
