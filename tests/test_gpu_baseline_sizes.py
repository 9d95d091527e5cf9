"""GPU (libsimmd through the C ABI) vs the CPU oracle at the sizes of the
reference configurations, FP64 path:

  * C1  3D LJ N = 1000, Newtonian NVE, dt = 0.01, skin 0.3, 10^4 steps.
        Strict over the first 200 steps (positions within 1e-9, velocities
        within 1e-8 box units, identical rebuild count); over 10^4 steps the
        trajectories decorrelate (two FP64 runs that differ only in the
        order of their force sums separate by ~13x per 50 steps and are
        fully independent after ~700 steps), so the long run is compared
        statistically: rebuild count within 2 %, mean E_tot/N over the
        second half within 5e-3, and the linear-fit drift of E_tot/N within
        0.05 per particle per 10^5 steps of the oracle's (the spread of the
        fitted drift between equivalent FP64 runs of the oracle is 3.4e-2).
  * C2  3D polydisperse soft spheres N = 32768, Langevin, host noise, 200
        steps: pair sets bit-exact, positions and velocities within 1e-11,
        identical rebuild count.
  * C3  the same system at N = 2^20: half and full pair sets bit-exact (the
        large-box test of the FP32 candidate classification), FP64 forces
        within 1e-12 of max |F|, energy and virial within 1e-12 relative.
  * C4  16 replicas of the 512-replica batch (2D and 3D, Brownian, Philox
        noise), FP64, advanced together in one batch for 50 steps: every
        replica within 1e-11 of the oracle's own run, same rebuild count.
Inputs are the seeded workloads of simulationcode_gb300.workloads; random
starts are relaxed first (capped steepest descent), and both sides start
from the same relaxed positions.
"""
import copy
import math

import numpy as np
import pytest

from gpu_helpers import GpuSystem, wrap_diff

pytestmark = pytest.mark.gpu


def _oracle_params(oracle, s, dynamics=None):
    return oracle.make_params(s.dims, s.potential, s.dynamics if dynamics is None else dynamics, s.N, s.box_size,
                              s.force_cutoff2, s.skin, eps=s.lj_eps, sigma=s.lj_sigma,
                              lj_rc=math.sqrt(s.force_cutoff2), zeta=s.b_zeta,
                              berthier_rc=math.sqrt(s.force_cutoff2), kBT=s.kBT, gamma=s.gamma, dt=s.dt, m=s.m)


def _pair_keys(N, counts, lst, both):
    """unordered pairs of an exported list as sorted int64 keys min*N+max"""
    rows = np.repeat(np.arange(N, dtype=np.int64), counts)
    mask = np.arange(lst.shape[1])[None, :] < counts[:, None]
    cols = lst[mask]
    keys = np.minimum(rows, cols) * N + np.maximum(rows, cols)
    keys.sort()
    if both:
        # each pair appears once from each side
        assert keys.size % 2 == 0 and np.array_equal(keys[0::2], keys[1::2])
        keys = keys[0::2]
    else:
        assert keys.size == 0 or np.all(keys[1:] != keys[:-1])  # each pair once
    return keys


def _gpu_keys(gpu, which, maxK):
    lib = gpu.lib
    from simulationcode_gb300 import _lib
    counts = np.zeros(gpu.N, np.int64)
    lst = np.zeros((gpu.N, maxK), np.int64)
    _lib.check(lib.simmd_export_pairs(gpu.ctx, which, maxK, _lib.ptr(counts), _lib.ptr(lst)))
    return _pair_keys(gpu.N, counts, lst - 1, both=(which == 1))


def _relaxed(specs):
    from simulationcode_gb300 import workloads as W
    W.relax_on_device(specs, 0)
    return specs


def test_c1_lj_nve_short_exact_long_statistical(simlib, oracle):
    from simulationcode_gb300 import workloads as W
    s = W.c1()[0]
    assert (s.N, s.dt, s.skin) == (1000, 0.01, 0.3)
    p = _oracle_params(oracle, s)
    ref = oracle.OracleSystem(p, s.r, s.D, v=s.v, force_cutoff=2.5)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, s.r, s.D, v=s.v, force_cutoff=2.5, tpp=8)
    gpu.rebuild()
    L = s.box_size
    # strict: 200 steps from the stale F = 0, as the reference's first step
    ref.run(200)
    gpu.step(200)
    rg, vg, _, _ = gpu.state()
    assert np.abs(wrap_diff(rg, ref.r, L)).max() < 1e-9
    assert np.abs(vg - ref.v).max() < 1e-8
    assert gpu.stats().rebuilds == ref.rebuilds
    # statistical: the rest of the 10^4 steps, E_tot/N every 100 steps
    e_ref, e_gpu = [], []
    for _ in range(98):
        ref.run(100)
        gpu.step(100)
        e_ref.append((ref.full_energy() + ref.kinetic_energy()) / s.N)
        ep, _, ek = gpu.energy()
        e_gpu.append((ep + ek) / s.N)
    steps = 200 + 100 * np.arange(1, 99)
    assert steps[-1] == 10 ** 4
    e_ref, e_gpu = np.array(e_ref), np.array(e_gpu)
    rb_ref, rb_gpu = ref.rebuilds, gpu.stats().rebuilds
    assert abs(rb_gpu - rb_ref) <= 0.02 * rb_ref, (rb_gpu, rb_ref)
    half = len(steps) // 2
    assert abs(e_gpu[half:].mean() - e_ref[half:].mean()) < 5e-3
    slope_ref = np.polyfit(steps, e_ref, 1)[0] * 1e5
    slope_gpu = np.polyfit(steps, e_gpu, 1)[0] * 1e5
    assert abs(slope_gpu - slope_ref) < 0.05, (slope_gpu, slope_ref)
    gpu.close()


def test_c2_soft_spheres_langevin_200_steps(simlib, oracle):
    from simulationcode_gb300 import workloads as W
    s = _relaxed(W.c2())[0]
    assert (s.N, s.dims, s.dt, s.skin) == (32768, 3, 0.005, 0.3)
    p = _oracle_params(oracle, s)
    ref = oracle.OracleSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, maxK=200)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, full_list=True)
    gpu.rebuild()
    N = s.N
    half_ref = _pair_keys(N, ref.nn_half, ref.list_half, both=False)
    full_ref = _pair_keys(N, ref.nn_full, ref.list_full, both=True)
    assert np.array_equal(_gpu_keys(gpu, 0, 200), half_ref)
    assert np.array_equal(_gpu_keys(gpu, 1, 200), full_ref)
    nsteps = 200
    noise = np.random.default_rng(12).standard_normal((nsteps, N, 3))
    ref.run(nsteps, noise=noise)
    gpu.step(nsteps, noise=noise)
    rg, vg, Fg, _ = gpu.state()
    assert np.abs(wrap_diff(rg, ref.r, s.box_size)).max() < 1e-11
    assert np.abs(vg - ref.v).max() < 1e-11
    assert np.abs(Fg - ref.F).max() < 1e-9 * np.abs(ref.F).max()
    assert gpu.stats().rebuilds == ref.rebuilds
    gpu.close()


def test_c3_pair_sets_and_forces_at_2_20(simlib, oracle):
    from simulationcode_gb300 import workloads as W
    s = _relaxed(W.c3())[0]
    assert s.N == 1 << 20 and abs(s.box_size - (s.N / 1.02) ** (1 / 3)) < 1e-9
    p = _oracle_params(oracle, s)
    maxK = 100
    ref = oracle.OracleSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, maxK=maxK)
    ref.update_neighbor_lists()
    N = s.N
    gpu = GpuSystem(p, s.r, s.D, v=s.v, force_cutoff=s.verlet_force_cutoff, full_list=True)
    gpu.rebuild()
    assert np.array_equal(_gpu_keys(gpu, 0, maxK), _pair_keys(N, ref.nn_half, ref.list_half, both=False))
    full_gpu = _gpu_keys(gpu, 1, maxK)
    full_ref = _pair_keys(N, ref.nn_full, ref.list_full, both=True)
    assert np.array_equal(full_gpu, full_ref)
    Fr = ref.calculate_new_forces().copy()
    Fg = gpu.forces()
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()
    e, w, _ = gpu.energy()
    assert e == pytest.approx(ref.full_energy(), rel=1e-12)
    assert w == pytest.approx(ref.virial(), rel=1e-12)
    gpu.close()


def test_c4_sixteen_batched_replicas_vs_oracle(simlib, oracle):
    from simulationcode_gb300 import _lib, workloads as W
    from simulationcode_gb300.batch import ReplicaBatch
    specs = W.c4(precision=_lib.FP64)[:16]
    assert {s.dims for s in specs} == {2, 3} and all(s.dynamics == _lib.BROWNIAN for s in specs)
    _relaxed(specs)
    nsteps = 50
    b = ReplicaBatch(0, tpp=1, graphs=True, graph_steps=16)
    ids = [b.add(copy.copy(s)) for s in specs]
    b.rebuild()
    b.step(nsteps)
    for rid, s in zip(ids, specs):
        p = _oracle_params(oracle, s)
        ref = oracle.OracleSystem(p, s.r, s.D, force_cutoff=s.verlet_force_cutoff, maxK=s.max_neighbors * 2)
        ref.update_neighbor_lists()
        ref.run(nsteps, seed=s.seed, step0=0)  # Philox noise keyed by (seed, step)
        rg = b.state(rid)[0]
        assert np.abs(wrap_diff(rg, ref.r, s.box_size)).max() < 1e-11, (rid, s.N, s.dims)
        assert b.stats(rid).rebuilds == ref.rebuilds  # both count the initial build
    b.close()
