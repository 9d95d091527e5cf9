"""The reference's MD driver (perform_molecular_dynamics!, src/MD.jl:680-719,
restated in simulationcode_gb300.md) run on the device through
NeighborListStruct, against the same driver run on the CPU oracle
(tests/oracle_nl.py), on a 1000-particle LJ system with a dump schedule
(save_data rebuilds the lists at every dump step, src/Dump.jl:64-67), a log
step (energy and the E_pot_test cross-check) and velocity randomisation,
short equilibration and rescale:

  * device vs oracle: final positions within 1e-10 and velocities within
    1e-9 (box units; 1000 steps of dt = 0.002 keep two FP64 trajectories
    within ~1e-13), the same dump steps with positions within 1e-10, the
    same N_neighbor_list_rebuilds, logged energies within 1e-12 relative,
    and the device's E_pot_test (lists built afresh) equal to the oracle's
    O(N^2) E_pot_test within 1e-12;
  * no-op callback (steps batched into few device calls) vs a per-step
    callback (every step a device call, state copied back each step):
    bit-identical final state, dumps and rebuild count.
"""
import numpy as np
import pytest

from cases import md_case
from gpu_helpers import wrap_diff
from oracle_nl import OracleNeighborList

pytestmark = pytest.mark.gpu


def _run(nl_factory, callback=None):
    from simulationcode_gb300 import md
    arrays, params, output, dumps = md_case(N=1000, N_steps=1000, N_eq=20, callback=callback)
    nl = nl_factory(params)
    logged = md.perform_molecular_dynamics_(arrays, params, output, nl, log=None)
    return arrays, params, output, dumps, logged, nl


def _gpu(params):
    from simulationcode_gb300 import md
    return md.initialize_neighbor_struct(0.3, params.box_size, 2.5, params.N, np.ones(params.N), 3)


def test_driver_device_vs_oracle_with_dumps_and_logs(simlib, oracle):
    a_o, params, out_o, dumps_o, log_o, _ = _run(lambda p: OracleNeighborList(0.3, 2.5))
    a_g, _, out_g, dumps_g, log_g, nl = _run(_gpu)
    L = params.box_size
    assert out_g.steps_done == out_o.steps_done == params.N_steps
    assert np.abs(wrap_diff(a_g.r_array, a_o.r_array, L)).max() < 1e-10
    assert np.abs(a_g.v_array - a_o.v_array).max() < 1e-9
    assert out_g.N_neighbor_list_rebuilds == out_o.N_neighbor_list_rebuilds
    assert sorted(dumps_g) == sorted(dumps_o) and len(dumps_g) > 10
    for t in dumps_o:
        assert np.abs(wrap_diff(dumps_g[t]["positions"], dumps_o[t]["positions"], L)).max() < 1e-10, t
        eg, eo = dumps_g[t]["potential_energy"], dumps_o[t]["potential_energy"]
        assert np.abs(eg - eo).max() <= 1e-10 * np.abs(eo).max(), t
    assert [x["step"] for x in log_g] == [x["step"] for x in log_o] == [1000]
    for xg, xo in zip(log_g, log_o):
        assert xg["E_pot"] == pytest.approx(xo["E_pot"], rel=1e-12)
        assert xg["E_pot_test"] == pytest.approx(xo["E_pot_test"], rel=1e-12)
        assert xg["E_pot_test"] == pytest.approx(xg["E_pot"], rel=1e-12)
        assert xg["E_kin"] == pytest.approx(xo["E_kin"], rel=1e-11)
    # batching: far fewer device step calls than steps (one per run of
    # steps between dump / log steps)
    assert nl.device_calls <= len(dumps_g) + 3


def test_driver_noop_callback_batches_bit_identically(simlib):
    calls = []
    a_b, _, out_b, dumps_b, _, nl_b = _run(_gpu)
    a_c, params, out_c, dumps_c, _, nl_c = _run(_gpu, callback=lambda a, p, o, nl: calls.append(o.steps_done))
    assert calls == list(range(params.N_steps + 1))
    assert nl_c.device_calls >= params.N_steps > 10 * nl_b.device_calls
    assert np.array_equal(a_b.r_array, a_c.r_array)
    assert np.array_equal(a_b.v_array, a_c.v_array)
    assert np.array_equal(a_b.F_array, a_c.F_array)
    assert out_b.N_neighbor_list_rebuilds == out_c.N_neighbor_list_rebuilds
    assert sorted(dumps_b) == sorted(dumps_c)
    for t in dumps_b:
        assert np.array_equal(dumps_b[t]["positions"], dumps_c[t]["positions"])
