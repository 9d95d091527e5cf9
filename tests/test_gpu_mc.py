"""Swap Monte Carlo on the device (simmd_mc_sweeps: do_MC_step! with
translation and swap moves, src/MC.jl:21-156) against the oracle's
restatement with the same keyed random draws: the same number of accepted
and tried moves of each kind, positions and diameters equal (each accepted
move is the same FP64 arithmetic; the energies behind the decisions differ
from the oracle's only in the order of the per-particle sums, ~1e-16), the
accumulated dE within 1e-10 relative, the same list rebuilds inside the
sweeps; and a replica's chain is the same alone and in a batch."""
import copy

import numpy as np
import pytest

from cases import make_case
from gpu_helpers import GpuSystem, wrap_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pot,dims,N,kBT", [(1, 3, 1728, 0.3), (1, 2, 1600, 0.3), (0, 3, 1000, 1.0)])
def test_mc_sweeps_match_oracle(simlib, oracle, pot, dims, N, kBT):
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=6, skin=0.6)
    p.kBT = kBT
    seed = 4242
    swap = 0.2 if pot == 1 else 0.0
    ref = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, force_cutoff=rc, full_list=True, seed=seed)
    gpu.rebuild()
    nsweeps, max_disp = 16, 0.12  # large enough moves that lists are rebuilt inside sweeps
    c_ref, de_ref = ref.mc_sweeps(nsweeps, max_disp, swap, seed=seed)
    from simulationcode_gb300 import _lib
    _lib.check(gpu.lib.simmd_mc_sweeps(gpu.ctx, nsweeps, max_disp, swap))
    counts = np.zeros(4, np.int64)
    import ctypes as C
    de = C.c_double()
    _lib.check(gpu.lib.simmd_mc_stats(gpu.ctx, 0, _lib.ptr(counts), C.byref(de)))
    Dg = np.zeros(N)
    _lib.check(gpu.lib.simmd_download_diameters(gpu.ctx, 0, _lib.ptr(Dg)))
    rg = gpu.state()[0]
    assert counts.tolist() == c_ref.tolist()
    assert counts[0] > 0 and (swap == 0 or counts[2] > 0)
    assert np.abs(wrap_diff(rg, ref.r, p.box_size)).max() <= 1e-12
    assert np.array_equal(Dg, ref.D)
    assert de.value == pytest.approx(de_ref, rel=1e-10)
    assert gpu.stats().rebuilds == ref.rebuilds > 1
    gpu.close()


def test_mc_replica_alone_equals_in_a_batch(simlib):
    from simulationcode_gb300 import _lib, workloads as W
    from simulationcode_gb300.batch import ReplicaBatch
    rng = np.random.default_rng(2)
    # the full Verlet list at skin 0.6 holds up to ~130 entries a particle
    specs = [W.berthier_spec(900, 2, _lib.BROWNIAN, rng, seed=31, skin=0.6, max_neighbors=200),
             W.berthier_spec(1300, 3, _lib.NEWTONIAN, rng, seed=32, skin=0.6, max_neighbors=200),
             W.lj_spec(1000, 3, _lib.LANGEVIN, rng, seed=33, skin=0.6, max_neighbors=200)]
    W.relax_on_device(specs, 0)
    mix = ReplicaBatch(0)
    ids = [mix.add(copy.copy(s)) for s in specs]
    mix.rebuild()
    mix.mc_sweeps(6, 0.05, 0.1)
    for rid, s in zip(ids, specs):
        alone = ReplicaBatch(0)
        a = alone.add(copy.copy(s))
        alone.rebuild()
        alone.mc_sweeps(6, 0.05, 0.1)
        assert np.array_equal(alone.state(a)[0], mix.state(rid)[0])
        assert np.array_equal(alone.diameters(a), mix.diameters(rid))
        ca, da = alone.mc_stats(a)
        cm, dm = mix.mc_stats(rid)
        assert ca.tolist() == cm.tolist() and da == dm
        alone.close()
    mix.close()


def test_mc_driver_device_vs_oracle(simlib, oracle):
    """perform_swap_monte_carlo! (restated in simulationcode_gb300.md) on the
    device list against the same driver on the oracle list: the same move
    counts, positions, diameters, dumps and kept energy; sweeps batched into
    few device calls with the no-op callback."""
    from cases import mc_case
    from oracle_nl import OracleNeighborList
    from simulationcode_gb300 import md
    a_o, params, out_o, dumps_o = mc_case(N=1000, N_steps=60)
    a_g, params_g, out_g, dumps_g = mc_case(N=1000, N_steps=60)  # its own dump writer
    log_o = md.perform_swap_monte_carlo_(a_o, params, out_o, OracleNeighborList(0.6, 1.25, seed=params.random_seed),
                                         log=None)
    nl = md.initialize_neighbor_struct(0.6, params.box_size, 1.25, params.N, a_g.D_array, 3)
    log_g = md.perform_swap_monte_carlo_(a_g, params_g, out_g, nl, log=None)
    for f in ("N_translations_accepted", "N_translations_total", "N_swaps_accepted", "N_swaps_total",
              "steps_done", "N_neighbor_list_rebuilds"):
        assert getattr(out_g, f) == getattr(out_o, f), f
    assert np.abs(wrap_diff(a_g.r_array, a_o.r_array, params.box_size)).max() <= 1e-12
    assert np.array_equal(a_g.D_array, a_o.D_array)
    assert out_g.potential_energy == pytest.approx(out_o.potential_energy, rel=1e-10)
    assert sorted(dumps_g) == sorted(dumps_o)
    for t in dumps_o:
        assert np.array_equal(dumps_g[t]["diameters"], dumps_o[t]["diameters"])
    assert [x["E_pot_test"] for x in log_g] == pytest.approx([x["E_pot_test"] for x in log_o], rel=1e-12)
    assert nl.device_calls <= len(dumps_g) + 2
