"""Split-precision error report: the FP32-split path beside the FP64 path on
the same system, run side by side as two replicas of one batch (they do not
interact; each is bit-identical to running alone).

Reported, per the three error figures of the split-precision contract:
  * force relative RMS  sqrt(sum|F32 - F64|^2 / sum|F64|^2) on identical
    configurations (the start, and the FP64 trajectory's state at the end);
  * |E32 - E64| / N  of the potential energy on those configurations;
  * the drift of E_tot/N per 1e5 steps of each run, from a linear fit of the
    sampled E_tot/N against the step (NVE, velocity Verlet,
    src/MD.jl:499-554), and of their difference.

Default workload: 3D polydisperse soft spheres, N = 2^20, rho = 1.02,
Newtonian NVE, dt = 0.005, Gaussian velocities at kBT = 0.1, 2e4 steps.

    python -m simulationcode_gb300.precision [--N 1048576] [--steps 20000] [--every 500]
"""
from __future__ import annotations

import argparse
import copy
import json
import math
import sys
import time

import numpy as np

from . import _lib
from . import workloads as W
from .batch import ReplicaBatch


def _forces_and_energy(spec, device, positions):
    """F (N x d) and E_pot of one configuration in both precisions"""
    out = {}
    for prec in (_lib.FP64, _lib.FP32_SPLIT):
        t = copy.copy(spec)
        t.r = positions
        t.precision = prec
        t.v = np.zeros_like(positions)
        b = ReplicaBatch(device)
        i = b.add(t)
        b.rebuild()
        _lib.check(b.lib.simmd_forces(b.ctx, None, None))
        en = b.energies()[i]
        out[prec] = (b.state(i)[2], en.epot)
        b.close()
    (f64, e64), (f32, e32) = out[_lib.FP64], out[_lib.FP32_SPLIT]
    rms = math.sqrt(float(((f32 - f64) ** 2).sum()) / float((f64 ** 2).sum()))
    return rms, abs(e32 - e64) / spec.N


def report(N=1 << 20, steps=20000, every=500, device=0, seed=3, relax_steps=300, log=None):
    rng = np.random.default_rng(seed)
    spec = W.berthier_spec(N, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=_lib.FP64, seed=seed)
    W.relax_on_device([spec], device, steps=relax_steps)
    rms0, de0 = _forces_and_energy(spec, device, spec.r)
    if steps <= 0:  # the relaxed start only
        return {"workload": "3D polydisperse soft spheres N=%d rho=1.02, relaxed start" % N,
                "force_rel_rms_start": rms0, "energy_abs_per_particle_start": de0,
                "bars": {"force_rel_rms": 1e-5}}
    s64 = copy.copy(spec)
    s32 = copy.copy(spec)
    s32.precision = _lib.FP32_SPLIT
    b = ReplicaBatch(device)
    i64, i32 = b.add(s64), b.add(s32)
    b.rebuild()
    t, e64, e32 = [], [], []
    t0 = time.perf_counter()
    for k in range(steps // every + 1):
        en = b.energies()
        t.append(k * every)
        e64.append((en[i64].epot + en[i64].ekin) / N)
        e32.append((en[i32].epot + en[i32].ekin) / N)
        if log:
            log("step %d  E/N fp64 %.9f  fp32 %.9f" % (t[-1], e64[-1], e32[-1]))
        if k < steps // every:
            b.step(every)
    wall = time.perf_counter() - t0
    r_end = b.state(i64)[0]
    st64, st32 = b.stats(i64), b.stats(i32)
    b.close()
    rms1, de1 = _forces_and_energy(spec, device, r_end)
    ta, a64, a32 = np.array(t, float), np.array(e64), np.array(e32)
    slope64 = float(np.polyfit(ta, a64, 1)[0]) * 1e5
    slope32 = float(np.polyfit(ta, a32, 1)[0]) * 1e5
    slope_d = float(np.polyfit(ta, a32 - a64, 1)[0]) * 1e5
    return {
        "workload": "3D polydisperse soft spheres N=%d rho=1.02, Newtonian NVE dt=0.005, kBT=0.1 start, "
                    "%d steps" % (N, steps),
        "force_rel_rms_start": rms0, "force_rel_rms_end": rms1,
        "energy_abs_per_particle_start": de0, "energy_abs_per_particle_end": de1,
        "drift_per_particle_per_1e5_steps_fp64": slope64,
        "drift_per_particle_per_1e5_steps_fp32_split": slope32,
        "drift_difference_per_1e5_steps": slope_d,
        "etot_per_particle_fp64": [float(x) for x in a64],
        "etot_per_particle_fp32_split": [float(x) for x in a32],
        "sample_every": every, "rebuilds_fp64": int(st64.rebuilds), "rebuilds_fp32_split": int(st32.rebuilds),
        "wall_s": wall,
        "bars": {"force_rel_rms": 1e-5, "drift_per_particle_per_1e5_steps": 1e-4},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--N", type=int, default=1 << 20)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--every", type=int, default=500)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--relax-steps", type=int, default=300)
    a = ap.parse_args()
    out = report(a.N, a.steps, a.every, a.device, relax_steps=a.relax_steps,
                 log=lambda m: print(m, file=sys.stderr, flush=True))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
