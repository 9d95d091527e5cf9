"""Edge cases of the CUDA path (FP64, through the C ABI) against the oracle.

  * One particle: no neighbours, zero force, energy and virial; a few
    Newtonian steps equal the oracle's (the centre-of-mass removal of
    src/MD.jl:532-541 stops the lone particle after its first drift).
  * Two particles interacting across the periodic boundary, one of them at
    the box edge 0.0 (LJ 3D, soft spheres 2D), in a replica of far fewer
    particles than one 128-slot tile: the pair is found, forces within
    1e-12 of max|F|, energy and virial relative 1e-12, 20 steps within
    1e-11 of the oracle's.
  * A list longer than max_neighbors: the reference's add_pair!
    (src/NeighborLists.jl:82-104) writes past the list's rows and raises a
    BoundsError; the rebuild here reports SIMMD_ERR_NEIGHBOR_OVERFLOW.  With
    the rows raised (simmd_reserve) and the positions uploaded again, the
    pair sets are the oracle's, bit for bit.
"""
import numpy as np
import pytest

from cases import make_case
from gpu_helpers import GpuSystem, wrap_diff
from simulationcode_gb300 import _lib

pytestmark = pytest.mark.gpu

LJ_RC, SOFT_RC = 2.5, 1.25


def _lj3(oracle, N, L):
    return oracle.make_params(3, oracle.POT_LJ, oracle.NEWTONIAN, N, L, LJ_RC ** 2, 0.3, eps=1.0, sigma=1.0,
                              lj_rc=LJ_RC, kBT=0.1, gamma=1.0, dt=0.005)


def test_single_particle(simlib, oracle):
    p = _lj3(oracle, 1, 10.0)
    r = np.array([[0.0, 5.0, 9.9999]])  # the first drift wraps x and z
    v = np.array([[-0.1, -0.2, 0.3]])
    D = np.ones(1)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=LJ_RC)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=LJ_RC)
    gpu.rebuild()
    assert np.array_equal(gpu.forces(), np.zeros((1, 3)))
    e, w, _ = gpu.energy()
    assert e == 0.0 and w == 0.0
    ref.run(5)
    gpu.step(5)
    r_g, v_g, _, _ = gpu.state()
    assert np.abs(wrap_diff(r_g, ref.r, 10.0)).max() <= 1e-12
    assert np.abs(v_g - ref.v).max() <= 1e-12
    gpu.close()


def _two_particle_case(oracle, which):
    if which == "lj3":
        L = 10.0
        p = _lj3(oracle, 2, L)
        r = np.array([[0.0, 5.0, 5.0], [9.2, 5.2, 4.9]])
        D = np.ones(2)
        return p, r, D, LJ_RC, L
    L = 6.0
    p = oracle.make_params(2, oracle.POT_BERTHIER, oracle.NEWTONIAN, 2, L, SOFT_RC ** 2, 0.3, zeta=0.2,
                           berthier_rc=SOFT_RC, kBT=0.1, gamma=1.0, dt=0.005)
    r = np.array([[0.0, 3.0], [5.2, 3.1]])
    D = np.array([0.8, 1.5])
    return p, r, D, SOFT_RC, L


@pytest.mark.parametrize("which", ["lj3", "soft2"])
def test_two_particles_across_the_boundary(simlib, oracle, which):
    p, r, D, rc, L = _two_particle_case(oracle, which)
    v = np.zeros_like(r)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    Fr = ref.calculate_new_forces().copy()
    assert np.abs(Fr).max() > 1.0  # the pair interacts
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc, full_list=True)
    gpu.rebuild()
    assert np.array_equal(gpu.pairs(0), ref.half_pairs())
    assert np.array_equal(gpu.pairs(1), ref.full_pairs())
    Fg = gpu.forces()
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()
    e, w, _ = gpu.energy()
    assert e == pytest.approx(ref.full_energy(), rel=1e-12)
    assert w == pytest.approx(ref.virial(), rel=1e-12)
    ref.run(20)
    gpu.step(20)
    r_g, v_g, _, _ = gpu.state()
    assert np.abs(wrap_diff(r_g, ref.r, L)).max() <= 1e-11
    assert np.abs(v_g - ref.v).max() <= 1e-11
    assert gpu.stats().rebuilds == ref.rebuilds
    gpu.close()


def test_list_overflow_reported_then_rows_raised(simlib, oracle):
    p, r, v, D, rc = make_case(1, 3, oracle.NEWTONIAN, 1728, seed=1)
    gpu = GpuSystem(p, r, D, force_cutoff=rc, full_list=True, max_neighbors=8)
    with pytest.raises(_lib.SimMDError) as err:
        gpu.rebuild()
    assert err.value.status == _lib.ERR_NEIGHBOR_OVERFLOW
    assert b"max_neighbors" in simlib.simmd_last_error()
    assert gpu.stats().overflow == 1
    # the user's remedy: more list rows, the neighbour structure set up again
    _lib.check(simlib.simmd_reserve(gpu.ctx, 0, 0, 0, 200))
    rr, DD = _lib.f64(r, (p.N, 3)), _lib.f64(D, (p.N,))
    _lib.check(simlib.simmd_upload(gpu.ctx, _lib.ptr(rr), None, None, _lib.ptr(DD), None))
    gpu.rebuild()
    assert gpu.stats().overflow == 0
    ref = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    ref.update_neighbor_lists()
    assert np.array_equal(gpu.pairs(0), ref.half_pairs())
    assert np.array_equal(gpu.pairs(1), ref.full_pairs())
    gpu.close()
