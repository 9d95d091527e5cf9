"""Generates the golden fixtures of tests/golden/*.npz from the oracle (the
serial C restatement of the reference's hot path under oracle/).

Each fixture freezes, for one small seeded system, the inputs (parameters,
r, v, D) and the oracle's outputs:
  * the half (force) and full (Verlet) neighbour pair sets,
  * forces with the host noise array given (Langevin/Brownian) or none,
    potential energy, per-particle energy, virial and kinetic energy,
  * the state after 12 steps driven by the Philox noise stream of ``seed``
    (r, v, F, displacement since the last rebuild, rebuild count).

The reference itself (Julia) cannot run here, so these pin the oracle and
the CUDA path against each other and against later changes, not against
the reference's own outputs.

    python tests/golden/make_golden.py      # from the repository root
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build as ob  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from cases import make_case  # noqa: E402

# name: (pot, dims, dyn, N, seed, dt)
CASES = {
    "lj3_newtonian": (O.POT_LJ, 3, O.NEWTONIAN, 216, 31, 0.005),
    "lj2_langevin": (O.POT_LJ, 2, O.LANGEVIN, 256, 32, 0.005),
    "berthier3_brownian": (O.POT_BERTHIER, 3, O.BROWNIAN, 343, 33, 2e-5),
    "berthier2_langevin": (O.POT_BERTHIER, 2, O.LANGEVIN, 300, 34, 0.005),
    "berthier3_newtonian": (O.POT_BERTHIER, 3, O.NEWTONIAN, 400, 35, 0.005),
}
PARAM_FIELDS = [f for f, _ in O.OrcParams._fields_]
PHILOX_SEED = 20240917
TRAJ_STEPS = 12


def params_json(p):
    return json.dumps({f: getattr(p, f) for f in PARAM_FIELDS})


def params_from_json(s):
    p = O.OrcParams()
    for k, v in json.loads(s).items():
        setattr(p, k, v)
    return p


def compute(p, r, v, D, rc, noise):
    """the oracle outputs of one fixture's inputs"""
    out = {}
    ref = O.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    out["half_pairs"] = ref.half_pairs().astype(np.int32)
    out["full_pairs"] = ref.full_pairs().astype(np.int32)
    out["F"] = ref.calculate_new_forces(noise).copy()
    out["epot"] = np.float64(ref.full_energy())
    out["epp"] = ref.per_particle_energy().copy()
    out["virial"] = np.float64(ref.virial())
    out["ekin"] = np.float64(ref.kinetic_energy())
    traj = O.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    traj.update_neighbor_lists()
    traj.run(TRAJ_STEPS, seed=PHILOX_SEED, step0=0)
    out["traj_r"] = traj.r.copy()
    out["traj_v"] = traj.v.copy()
    out["traj_F"] = traj.F.copy()
    out["traj_disp"] = traj.disp.copy()
    out["traj_rebuilds"] = np.int64(traj.rebuilds)
    return out


def inputs(name):
    pot, dims, dyn, N, seed, dt = CASES[name]
    p, r, v, D, rc = make_case(pot, dims, dyn, N, seed=seed, dt=dt)
    if v is None:
        v = np.zeros((N, dims))
    noise = O.philox_normals(PHILOX_SEED + 1, 0, N, dims) if dyn != O.NEWTONIAN else None
    return p, r, v, D, rc, noise


def main():
    ob.build_oracle()
    for name in CASES:
        p, r, v, D, rc, noise = inputs(name)
        out = compute(p, r, v, D, rc, noise)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), params=np.array(params_json(p)), r=r, v=v, D=D,
                            rc=np.float64(rc), noise=noise if noise is not None else np.zeros((0,)),
                            philox_seed=np.int64(PHILOX_SEED), traj_steps=np.int64(TRAJ_STEPS), **out)
        print(name, "N=%d" % p.N, "half pairs %d" % len(out["half_pairs"]),
              "rebuilds %d" % out["traj_rebuilds"])


if __name__ == "__main__":
    main()
