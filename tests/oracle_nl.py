"""A neighbour-list object backed by the CPU oracle, with the methods that
simulationcode_gb300.md's generic functions dispatch to (test
infrastructure: it lets the reference's MD driver, as restated in
simulationcode_gb300.md, run unchanged on the oracle, so that a device run
and an oracle run of the same driver can be compared step for step).

The oracle keeps its own copies of r, v, F and the displacement; they are
synchronised with the ArrayStruct around every call, as the reference's
functions read and write the ArrayStruct fields directly.
"""
from __future__ import annotations

import math

import numpy as np

from oracle import pyoracle as O
from simulationcode_gb300.structs import Berthier, Brownian, Langevin, LJ, Newtonian


def oracle_params(parameters, skin):
    s, U = parameters.system, parameters.interaction_potential
    dyn = O.NEWTONIAN if isinstance(s, Newtonian) else (O.LANGEVIN if isinstance(s, Langevin) else O.BROWNIAN)
    kw = dict(kBT=s.kBT, dt=s.dt, gamma=getattr(s, "gamma", 1.0), m=getattr(s, "m", 1.0),
              rescale=bool(getattr(s, "rescale_temperature", False)))
    if isinstance(U, LJ):
        return O.make_params(s.dims, O.POT_LJ, dyn, parameters.N, parameters.box_size, parameters.force_cutoff2,
                             skin, eps=U.eps, sigma=U.sigma, lj_rc=U.rc, **kw)
    assert isinstance(U, Berthier)
    return O.make_params(s.dims, O.POT_BERTHIER, dyn, parameters.N, parameters.box_size, parameters.force_cutoff2,
                         skin, zeta=U.zeta, berthier_rc=U.rc, **kw)


class OracleNeighborList:
    """NeighborListStruct stand-in running every computation in the oracle;
    random forces from the oracle's Philox stream keyed by (seed, step)."""

    def __init__(self, skin_distance, force_cutoff, maxneighbours=200, seed=1):
        self.skin_distance = float(skin_distance)
        self.force_cutoff = float(force_cutoff)
        self.maxneighbours = int(maxneighbours)
        self.seed = int(seed)
        self.sys = None
        self.noise_step = 0
        self.mc_sweep = 0
        self._rebuilds_seen = 0

    def _ensure(self, arrays, parameters):
        if self.sys is None:
            p = oracle_params(parameters, self.skin_distance)
            self.sys = O.OracleSystem(p, arrays.r_array, arrays.D_array, v=arrays.v_array, F=arrays.F_array,
                                      maxK=self.maxneighbours, force_cutoff=self.force_cutoff)

    def _in(self, arrays, parameters):
        self._ensure(arrays, parameters)
        self.sys.r[:] = arrays.r_array
        self.sys.v[:] = arrays.v_array
        self.sys.F[:] = arrays.F_array
        self.sys.D[:] = arrays.D_array

    def _out(self, arrays, output):
        arrays.r_array[:] = self.sys.r
        arrays.v_array[:] = self.sys.v
        arrays.F_array[:] = self.sys.F
        arrays.D_array[:] = self.sys.D
        if output is not None:
            output.N_neighbor_list_rebuilds += self.sys.rebuilds - self._rebuilds_seen
        self._rebuilds_seen = self.sys.rebuilds

    def update_neighbor_lists_(self, arrays, parameters, output):
        self._in(arrays, parameters)
        self.sys.update_neighbor_lists()
        self._out(arrays, output)

    def do_time_step(self, arrays, parameters, output, system, noise=None, nsteps=1):
        self._in(arrays, parameters)
        if noise is not None:
            self.sys.run(nsteps, noise=np.asarray(noise).reshape(nsteps, parameters.N, system.dims))
        else:
            self.sys.run(nsteps, seed=self.seed, step0=self.noise_step)
            if not isinstance(system, Newtonian):
                self.noise_step += nsteps
        self._out(arrays, output)

    def do_MC_step_(self, arrays, parameters, output, swap_probability):
        self._in(arrays, parameters)
        counts, de = self.sys.mc_sweeps(1, parameters.max_MC_displacement, swap_probability, self.seed,
                                        sweep0=self.mc_sweep)
        self.mc_sweep += 1
        output.N_translations_accepted += int(counts[0])
        output.N_translations_total += int(counts[1])
        output.N_swaps_accepted += int(counts[2])
        output.N_swaps_total += int(counts[3])
        output.potential_energy += de
        self._out(arrays, output)

    def run_short_MD_equilibration_(self, arrays, parameters, output):
        self.update_neighbor_lists_(arrays, parameters, output)
        for _ in range(parameters.N_MD_equilibration_steps):
            self.do_time_step(arrays, parameters, output, parameters.system)

    def calculate_new_forces_(self, arrays, parameters, noise=None):
        self._in(arrays, parameters)
        self.sys.calculate_new_forces(noise)
        self._out(arrays, None)

    def calculate_full_energy(self, arrays, parameters):
        self._in(arrays, parameters)
        return self.sys.full_energy()

    def calculate_virial(self, arrays, parameters):
        self._in(arrays, parameters)
        return self.sys.virial()

    def compute_potential_energy_(self, arrays, parameters, output):
        self._in(arrays, parameters)
        arrays.potential_energy_array[:] = self.sys.per_particle_energy()

    def calculate_full_energy_no_neigh(self, arrays, parameters):
        self._in(arrays, parameters)
        return self.sys.energy_no_neigh()  # the reference's O(N^2) E_pot_test
