"""The CUDA path (FP64, through the C ABI) against the committed golden
fixtures: pair sets bit-exact; forces within 1e-12 of max|F|; potential
energy, virial and kinetic energy within 1e-12 relative; per-particle
energies within 1e-12 of the largest; the 12-step Philox-noise trajectory
within 1e-11 (positions, box units; velocities) and 1e-9 of max|F| for
forces, with the same rebuild count."""
import glob
import os

import numpy as np
import pytest

from gpu_helpers import GpuSystem, wrap_diff

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def _fixture(path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    g = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(g)
    z = np.load(path)
    f = {k: z[k] for k in z.files}
    return g.params_from_json(str(f["params"])), f


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_matches_fixture(simlib, path):
    p, f = _fixture(path)
    rc = float(f["rc"])
    noise = f["noise"] if f["noise"].size else None
    v = f["v"] if p.dynamics != 2 else None
    gpu = GpuSystem(p, f["r"], f["D"], v=v, force_cutoff=rc, full_list=True)
    gpu.rebuild()
    assert np.array_equal(gpu.pairs(0).astype(np.int32), f["half_pairs"])
    assert np.array_equal(gpu.pairs(1).astype(np.int32), f["full_pairs"])
    F = gpu.forces(noise)
    assert np.abs(F - f["F"]).max() <= 1e-12 * np.abs(f["F"]).max()
    e, w, k = gpu.energy()
    assert _rel(e, float(f["epot"])) <= 1e-12
    assert _rel(w, float(f["virial"])) <= 1e-12
    if p.dynamics != 2:
        assert _rel(k, float(f["ekin"])) <= 1e-12
    epp = gpu.per_particle_energy()
    assert np.abs(epp - f["epp"]).max() <= 1e-12 * np.abs(f["epp"]).max()
    gpu.close()

    traj = GpuSystem(p, f["r"], f["D"], v=v, force_cutoff=rc, seed=int(f["philox_seed"]))
    traj.rebuild()
    traj.step(int(f["traj_steps"]))
    r, vv, FF, u = traj.state()
    assert np.abs(wrap_diff(r, f["traj_r"], p.box_size)).max() < 1e-11
    if p.dynamics != 2:
        assert np.abs(vv - f["traj_v"]).max() < 1e-11 * max(1.0, np.abs(f["traj_v"]).max())
    assert np.abs(FF - f["traj_F"]).max() <= 1e-9 * np.abs(f["traj_F"]).max()
    assert np.abs(u - f["traj_disp"]).max() < 1e-11
    assert traj.stats().rebuilds == int(f["traj_rebuilds"])
    traj.close()
