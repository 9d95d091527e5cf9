"""The restated reference driver (perform_molecular_dynamics!, src/MD.jl:680-719,
with save_data's dump-step rebuild, src/Dump.jl:64-67) run on the CPU oracle
through the generic functions of simulationcode_gb300.md, against the same
sequence of oracle calls written out by hand: velocity randomisation,
lists, short equilibration and rescale, then per step do_time_step, the
callback, a list rebuild at every dump step and the log-step energies.
Bit for bit (same oracle, same order of operations)."""
import math

import numpy as np

from cases import md_case
from oracle_nl import OracleNeighborList, oracle_params


def test_driver_on_oracle_matches_hand_written_sequence(oracle):
    from simulationcode_gb300 import md
    calls = []
    arrays, params, output, dumps = md_case(N=216, N_steps=1000, N_eq=10,
                                            callback=lambda a, p, o, nl: calls.append(o.steps_done))
    r0 = arrays.r_array.copy()
    nl = OracleNeighborList(0.3, 2.5)
    logged = md.perform_molecular_dynamics_(arrays, params, output, nl, log=None)
    # the same sequence by hand
    rng = np.random.default_rng(params.random_seed)
    v = rng.standard_normal(r0.shape) * math.sqrt(0.1 / 1.0)
    ref = oracle.OracleSystem(oracle_params(params, 0.3), r0, arrays.D_array, v=v, force_cutoff=2.5)
    ref.update_neighbor_lists()                      # perform_molecular_dynamics!
    ref.update_neighbor_lists()                      # run_short_MD_equilibration!
    ref.run(params.N_MD_equilibration_steps)
    md.rescale_velocities_(ref.v, params)
    rb0 = ref.rebuilds
    when = set(params.dump_info.when_to_save_array)
    assert 0 in when
    ref.update_neighbor_lists()                      # save_data at step 0
    hand_dumps, hand_log = {0: ref.r.copy()}, []
    for t in range(1, params.N_steps + 1):
        ref.run(1)
        if t in when:
            ref.update_neighbor_lists()
            hand_dumps[t] = ref.r.copy()
        if md.logdata(t):
            hand_log.append((t, ref.full_energy(), ref.energy_no_neigh()))
    assert np.array_equal(arrays.r_array, ref.r) and np.array_equal(arrays.v_array, ref.v)
    assert output.steps_done == params.N_steps
    assert output.N_neighbor_list_rebuilds == ref.rebuilds - rb0
    assert sorted(dumps) == sorted(hand_dumps)
    for t, d in dumps.items():
        assert np.array_equal(d["positions"], hand_dumps[t])
    assert calls == list(range(params.N_steps + 1))
    assert [(x["step"], x["E_pot"], x["E_pot_test"]) for x in logged] == hand_log
    assert [x[0] for x in hand_log] == [1000]


def test_logdata_and_dump_schedule():
    from simulationcode_gb300 import md
    assert md.logdata(0) and not md.logdata(1) and not md.logdata(999)
    assert md.logdata(1000) and md.logdata(2000) and not md.logdata(2500) and md.logdata(10 ** 5)
    w = md.create_when_to_save_array(1.5, 2, 100)
    # start times 0, 50, 100; from each t = 1, 2, 3, 5, 8, 12, 18, 27, 41, 62, 93 (x1.5, ceil)
    assert w[:8] == [0, 1, 2, 3, 5, 8, 12, 18] and w[-1] == 100 and 51 in w and 100 in w
    assert w == sorted(set(w)) and max(w) == 100
