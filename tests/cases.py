"""Seeded synthetic systems shared by the oracle and GPU tests.

Shapes and value distributions follow the reference's workloads: LJ at
rho = 1 on a jittered simple-cubic lattice (eps = sigma = 1, rc = 2.5) and
polydisperse Berthier soft spheres (D ~ P(D) ∝ D^-3 on [0.7253, 1.6095],
zeta = 0.2, rc = 1.25) at rho = 1.02 relaxed by the oracle's restatement of
find_random_initial_configuration! (MC at kBT = 10).
"""
from __future__ import annotations

import math

import numpy as np

from oracle import pyoracle as O


def lattice_positions(N, dims, L, jitter, rng):
    n = int(round(N ** (1.0 / dims)))
    assert n ** dims == N
    a = L / n
    g = np.stack(np.meshgrid(*([np.arange(n)] * dims), indexing="ij"), -1).reshape(-1, dims).astype(float)
    r = (g + 0.5) * a + rng.uniform(-jitter, jitter, (N, dims))
    return np.mod(r, L)


def make_case(pot, dims, dyn, N, *, rho=None, skin=0.3, seed=0, mc_sweeps=40, dt=None, kBT=0.1, gamma=1.0,
              jitter=0.05, vel=True):
    """Returns (oracle params, r, v, D, force_cutoff) for a seeded system."""
    rng = np.random.default_rng(seed)
    if pot == O.POT_LJ:
        rho = 1.0 if rho is None else rho
        L = (N / rho) ** (1.0 / dims)
        rc = 2.5
        D = np.ones(N)
        p = O.make_params(dims, O.POT_LJ, dyn, N, L, rc * rc, skin, eps=1.0, sigma=1.0, lj_rc=rc, kBT=kBT,
                          gamma=gamma, dt=dt or 0.005)
        n = int(round(N ** (1.0 / dims)))
        if n ** dims == N:
            r = lattice_positions(N, dims, L, jitter, rng)
        else:
            r = rng.uniform(0, L, (N, dims))
    else:
        rho = 1.02 if rho is None else rho
        L = (N / rho) ** (1.0 / dims)
        rc = 1.25
        D = O.generate_diameters_berthier(N, 2.219, seed + 11)
        p = O.make_params(dims, O.POT_BERTHIER, dyn, N, L, rc * rc, skin, zeta=0.2, berthier_rc=rc, kBT=kBT,
                          gamma=gamma, dt=dt or 0.005)
        if mc_sweeps > 0:
            r, _ = O.random_initial_configuration(p, D, mc_sweeps, max_disp=0.1, seed=seed + 5, skin=0.6)
        else:
            r = rng.uniform(0, L, (N, dims))
    v = None
    if vel and dyn != O.BROWNIAN:
        v = rng.standard_normal((N, dims)) * math.sqrt(kBT)
        v -= v.mean(0)
    return p, r, v, D, rc


def md_case(N=1000, dims=3, *, dt=0.002, N_steps=1000, N_eq=20, log_factor=1.5, N_starts=2, seed=3,
            callback=None):
    """(arrays, parameters, output, dumps) of an LJ system (rho = 1,
    jittered simple lattice, eps = sigma = 1, rc = 2.5, Newtonian) set up
    through the reference's structs for perform_molecular_dynamics!, with a
    dump schedule from create_when_to_save_array whose writer records every
    dump into ``dumps``"""
    from simulationcode_gb300 import md
    from simulationcode_gb300.structs import ArrayStruct, DumpInfo, LJ, Newtonian, OutputStruct, ParameterStruct
    rng = np.random.default_rng(seed)
    L = float(N) ** (1.0 / dims)
    U = LJ(1.0, 1.0, 2.5)
    dumps = {}
    di = DumpInfo(True, "unused.h5", md.create_when_to_save_array(log_factor, N_starts, N_steps),
                  save_r=True, save_v=True, save_F=True, save_Epot=True,
                  writer=lambda step, d: dumps.__setitem__(step, d))
    params = ParameterStruct(N_eq, seed, 1.0, N, L, N_steps, 0.0, 0.1, U.rc ** 2, 0.0,
                             Newtonian(0.1, dt, 1.0, False, dims), U, dump_info=di, callback=callback)
    arrays = ArrayStruct(N, dims)
    arrays.r_array[:] = lattice_positions(N, dims, L, 0.05, rng)
    arrays.D_array[:] = 1.0
    return arrays, params, OutputStruct(), dumps


def mc_case(N=1000, *, N_steps=50, log_factor=2.0, N_starts=1, seed=7, kBT=0.3, swap=0.2, max_disp=0.05,
            callback=None):
    """(arrays, parameters, output, dumps) of a 3D polydisperse soft-sphere
    system set up through the reference's structs for
    perform_swap_monte_carlo!: random positions relaxed by the oracle's
    initial-configuration MC, Berthier diameters, a dump schedule"""
    from simulationcode_gb300 import md
    from simulationcode_gb300.structs import ArrayStruct, Berthier, DumpInfo, Newtonian, OutputStruct, ParameterStruct
    p, r, v, D, rc = make_case(O.POT_BERTHIER, 3, O.NEWTONIAN, N, seed=seed, skin=0.6)
    U = Berthier()
    dumps = {}
    di = DumpInfo(True, "unused.h5", md.create_when_to_save_array(log_factor, N_starts, N_steps),
                  save_r=True, save_v=False, save_F=False, save_D=True,
                  writer=lambda step, d: dumps.__setitem__(step, d))
    params = ParameterStruct(0, seed, 1.02, N, p.box_size, N_steps, swap, max_disp, U.rc ** 2, 0.0,
                             Newtonian(kBT, 0.005, 1.0, False, 3), U, dump_info=di, callback=callback)
    arrays = ArrayStruct(N, 3)
    arrays.r_array[:] = r
    arrays.D_array[:] = D
    return arrays, params, OutputStruct(), dumps
