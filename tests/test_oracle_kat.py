"""Known-answer tests that pin the CPU oracle (no GPU needed).

The reference ships no tests or golden vectors, so the oracle is pinned by
analytic facts of the potentials and by invariants of the algorithms.
"""
import math

import numpy as np
import pytest

from cases import make_case


def test_berthier_constants_match_closed_form(oracle):
    c0, c2, c4 = oracle.berthier_constants(12, 1.25)
    assert c0 == pytest.approx(-28 / 1.25 ** 12, rel=1e-15)
    assert c2 == pytest.approx(48 / 1.25 ** 14, rel=1e-15)
    assert c4 == pytest.approx(-21 / 1.25 ** 16, rel=1e-15)


@pytest.mark.parametrize("s", [0.8, 1.0, 1.3])
def test_berthier_potential_and_force_vanish_at_cutoff(oracle, s):
    p = oracle.make_params(3, oracle.POT_BERTHIER, oracle.NEWTONIAN, 2, 10.0, 1.25 ** 2, 0.3)
    L = oracle.lib()
    md2 = s * s
    r2 = 1.25 ** 2 * md2
    import ctypes as C
    V = L.orc_pair_potential(C.byref(p), r2, md2)
    F = L.orc_pair_force(C.byref(p), r2, md2)
    assert abs(V) < 1e-13
    assert abs(F) < 1e-12
    # V(r -> 0.9 rc s) > 0 and force repulsive
    assert L.orc_pair_potential(C.byref(p), 0.8 * r2, md2) > 0
    assert L.orc_pair_force(C.byref(p), 0.5 * r2, md2) > 0


def test_lj_force_zero_at_minimum(oracle):
    import ctypes as C
    p = oracle.make_params(3, oracle.POT_LJ, oracle.NEWTONIAN, 2, 10.0, 6.25, 0.3)
    L = oracle.lib()
    rmin2 = 2 ** (1 / 3)
    assert abs(L.orc_pair_force(C.byref(p), rmin2, 1.0)) < 1e-13
    assert L.orc_pair_potential(C.byref(p), rmin2, 1.0) == pytest.approx(-1.0 - p.lj_Uc, abs=1e-14)
    # shifted potential vanishes at rc
    assert abs(L.orc_pair_potential(C.byref(p), 6.25, 1.0)) < 1e-15


def test_two_particle_lj_force(oracle):
    N, L = 2, 10.0
    p = oracle.make_params(3, oracle.POT_LJ, oracle.NEWTONIAN, N, L, 6.25, 0.3)
    r = np.array([[1.0, 1.0, 1.0], [2.3, 1.0, 1.0]])
    s = oracle.OracleSystem(p, r, np.ones(N))
    s.update_neighbor_lists()
    F = s.calculate_new_forces()
    x = 1.3
    fr = 48 / x ** 13 - 24 / x ** 7
    assert F[0, 0] == pytest.approx(-fr, rel=1e-14)
    assert F[1, 0] == pytest.approx(fr, rel=1e-14)
    # across the periodic boundary
    r2 = np.array([[0.2, 5.0, 5.0], [9.5, 5.0, 5.0]])
    s2 = oracle.OracleSystem(p, r2, np.ones(N))
    s2.update_neighbor_lists()
    F2 = s2.calculate_new_forces()
    x = 0.7
    fr = 48 / x ** 13 - 24 / x ** 7
    assert F2[0, 0] == pytest.approx(fr, rel=1e-13)


@pytest.mark.parametrize("pot,dims", [(0, 3), (1, 3), (1, 2), (0, 2)])
def test_cell_list_pairs_equal_all_pairs(oracle, pot, dims):
    N = 512 if dims == 3 else 576
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=3, mc_sweeps=5)
    a = oracle.OracleSystem(p, r, D, use_cells=True, force_cutoff=rc)
    b = oracle.OracleSystem(p, r, D, use_cells=False, force_cutoff=rc)
    a.update_neighbor_lists()
    b.update_neighbor_lists()
    assert np.array_equal(a.half_pairs(), b.half_pairs())
    assert np.array_equal(a.full_pairs(), b.full_pairs())
    assert a.full_energy() == pytest.approx(b.full_energy(), rel=1e-12)


@pytest.mark.parametrize("pot,dims", [(0, 3), (1, 3), (1, 2), (0, 2)])
def test_newton_third_law_and_energy_vs_brute_force(oracle, pot, dims):
    N = 343 if dims == 3 else 400
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=1, mc_sweeps=5)
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    F = s.calculate_new_forces()
    scale = np.abs(F).max()
    assert np.abs(F.sum(0)).max() < 1e-12 * scale * N
    assert s.full_energy() == pytest.approx(s.energy_no_neigh(), rel=1e-12)


@pytest.mark.parametrize("pot,dims", [(0, 3), (1, 3), (1, 2)])
def test_force_is_minus_energy_gradient(oracle, pot, dims):
    N = 216 if dims == 3 else 256
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=2, mc_sweeps=10)
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    F = s.pair_forces()
    rng = np.random.default_rng(0)
    for i in rng.choice(N, 5, replace=False):
        for k in range(dims):
            h = 1e-6
            s.r[i, k] += h
            ep = s.energy_no_neigh()
            s.r[i, k] -= 2 * h
            em = s.energy_no_neigh()
            s.r[i, k] += h
            g = -(ep - em) / (2 * h)
            assert F[i, k] == pytest.approx(g, rel=1e-5, abs=1e-6 * max(1.0, abs(F[i, k])))


@pytest.mark.parametrize("pot,dims", [(0, 3), (1, 3), (1, 2)])
def test_virial_is_minus_dE_dlambda(oracle, pot, dims):
    N = 216 if dims == 3 else 256
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=4, mc_sweeps=10)
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    W = s.virial()

    def energy(lam):
        q = oracle.OrcParams.from_buffer_copy(p)
        q.box_size = p.box_size * lam
        t = oracle.OracleSystem(q, r * lam, D, force_cutoff=rc)
        return t.energy_no_neigh()

    h = 1e-6
    dE = (energy(1 + h) - energy(1 - h)) / (2 * h)
    assert W == pytest.approx(-dE, rel=1e-5)


def test_newtonian_energy_conservation_lj(oracle):
    p, r, v, D, rc = make_case(0, 3, oracle.NEWTONIAN, 1000, seed=7, dt=0.005)
    s = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    s.update_neighbor_lists()
    s.calculate_new_forces()
    s.run(100)  # past the O(dt^2) transient of the lattice start
    e0 = s.full_energy() + s.kinetic_energy()
    s.run(300)
    e1 = s.full_energy() + s.kinetic_energy()
    assert abs(e1 - e0) / 1000 < 1e-3


def test_philox_known_answer(oracle):
    # Random123 known-answer vectors for philox4x32-10
    assert list(oracle.philox4x32_10([0, 0, 0, 0], [0, 0])) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert list(oracle.philox4x32_10([0xffffffff] * 4, [0xffffffff] * 2)) == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert list(oracle.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                     [0xa4093822, 0x299f31d0])) == [0xd16cfe09, 0x94fdcceb, 0x5001e420,
                                                                     0x24126ea1]


def test_philox_normals_statistics(oracle):
    z = oracle.philox_normals(1234, 7, 200000, 3)
    assert abs(z.mean()) < 0.01
    assert z.std() == pytest.approx(1.0, abs=0.01)
    z2 = oracle.philox_normals(1234, 8, 200000, 3)
    assert abs(np.corrcoef(z.ravel(), z2.ravel())[0, 1]) < 0.01


def test_diameters_support_and_mean(oracle):
    D = oracle.generate_diameters_berthier(100000, 2.219, 1)
    assert D.min() == pytest.approx(0.72533, abs=1e-4)
    assert D.max() == pytest.approx(1.60946, abs=1e-3)
    assert D.mean() == pytest.approx(1.0, abs=5e-3)


def test_brownian_removes_mean_force_and_langevin_runs(oracle):
    p, r, v, D, rc = make_case(1, 2, oracle.BROWNIAN, 400, seed=9, dt=1e-3)
    s = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    s.update_neighbor_lists()
    noise = np.random.default_rng(0).standard_normal((400, 2))
    s.step(noise)
    assert np.abs(s.F.sum(0)).max() < 1e-9 * np.abs(s.F).max() * 400
    p2, r2, v2, D2, rc2 = make_case(1, 3, oracle.LANGEVIN, 343, seed=9)
    s2 = oracle.OracleSystem(p2, r2, D2, v=v2, force_cutoff=rc2)
    s2.update_neighbor_lists()
    s2.run(20, seed=5)
    assert np.isfinite(s2.r).all() and np.abs(s2.v.mean(0)).max() < 1e-14
