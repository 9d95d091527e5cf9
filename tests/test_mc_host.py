"""The oracle's restatement of swap Monte Carlo (do_MC_step! with
do_translation_step! and do_swap_step!, src/MC.jl:21-156), checked for the
invariants the reference's own log line checks (E_pot kept by adding each
accepted move's dE equals the recomputed energy, src/MC.jl:196-221) and for
what a swap move must preserve (the multiset of diameters)."""
import numpy as np
import pytest

from cases import make_case


@pytest.mark.parametrize("pot,dims,N", [(1, 3, 512), (1, 2, 400), (0, 3, 216)])
def test_mc_energy_bookkeeping_and_swaps(oracle, pot, dims, N):
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=4, skin=0.6)
    p.kBT = 0.5
    o = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    o.update_neighbor_lists()
    e0 = o.full_energy()
    d0 = np.sort(o.D.copy())
    counts, de = o.mc_sweeps(10, 0.05, 0.2 if pot == 1 else 0.0, seed=99)
    e1 = o.full_energy()
    assert e0 + de == pytest.approx(e1, rel=1e-10, abs=1e-9)
    assert np.array_equal(np.sort(o.D), d0)
    assert counts[1] + (counts[3] if pot == 1 else 0) <= 10 * N
    assert 0 < counts[0] < counts[1]
    if pot == 1:
        assert counts[3] > 0 and counts[2] <= counts[3]
    assert np.all((o.r >= 0) & (o.r < p.box_size))


def test_mc_uniforms_are_keyed(oracle):
    a = oracle.mc_uniforms(5, 3, 17)
    assert np.all((a >= 0) & (a < 1)) and len(set(a.tolist())) == 6
    assert np.array_equal(a, oracle.mc_uniforms(5, 3, 17))
    assert not np.array_equal(a, oracle.mc_uniforms(5, 4, 17))
    assert not np.array_equal(a, oracle.mc_uniforms(6, 3, 17))


def test_mc_driver_on_oracle_matches_hand_written_sequence(oracle):
    """perform_swap_monte_carlo! as restated in simulationcode_gb300.md, run on
    the oracle-backed list, equals the same sequence of oracle calls written
    out: lists, per sweep do_MC_step!, a rebuild at every dump step, energy
    kept by the accepted dE."""
    from cases import mc_case
    from oracle_nl import OracleNeighborList, oracle_params
    from simulationcode_gb300 import md
    arrays, params, output, dumps = mc_case(N=216, N_steps=30)
    r0, D0 = arrays.r_array.copy(), arrays.D_array.copy()
    nl = OracleNeighborList(0.6, 1.25, seed=params.random_seed)
    md.perform_swap_monte_carlo_(arrays, params, output, nl, log=None)
    ref = oracle.OracleSystem(oracle_params(params, 0.6), r0, D0, force_cutoff=1.25)
    ref.update_neighbor_lists()
    when = set(params.dump_info.when_to_save_array)
    ref.update_neighbor_lists()            # save_data at step 0
    e = ref.energy_no_neigh()
    counts = np.zeros(4, np.int64)
    for t in range(params.N_steps + 1):
        c, de = ref.mc_sweeps(1, params.max_MC_displacement, params.swap_probability, params.random_seed, sweep0=t)
        counts += c
        e += de
        if t + 1 in when:
            ref.update_neighbor_lists()
    assert np.array_equal(arrays.r_array, ref.r) and np.array_equal(arrays.D_array, ref.D)
    assert [output.N_translations_accepted, output.N_translations_total, output.N_swaps_accepted,
            output.N_swaps_total] == counts.tolist()
    assert output.potential_energy == e
    assert output.steps_done == params.N_steps + 1
    assert output.potential_energy == pytest.approx(ref.energy_no_neigh(), rel=1e-10)
