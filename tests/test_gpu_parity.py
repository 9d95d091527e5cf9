"""GPU (libsimmd through the C ABI) vs the CPU oracle on the same seeded
inputs.  Tolerances (the FP64 path):
  * neighbour pair sets: bit-exact (identical unordered pair sets);
  * forces: max_i |F_gpu - F_ref| <= 1e-12 * max_i |F_ref|;
  * potential energy, virial: relative 1e-12;
  * trajectories (host-supplied noise): positions/velocities within
    1e-11 (absolute, box units) after the stated number of steps, and the
    same rebuild count.
The split-precision path: force relative RMS <= 1e-5 against FP64.
"""
import numpy as np
import pytest

from cases import make_case
from gpu_helpers import GpuSystem, wrap_diff

pytestmark = pytest.mark.gpu

CASES = [  # (pot, dims, N)
    (0, 3, 1000),   # LJ 3D, the small reference configuration
    (1, 3, 1728),   # Berthier 3D
    (1, 2, 1600),   # Berthier 2D
    (0, 2, 900),    # LJ 2D (generic path)
]


def _systems(oracle, pot, dims, dyn, N, seed=0, **kw):
    p, r, v, D, rc = make_case(pot, dims, dyn, N, seed=seed, **kw)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc, **{k: v_ for k, v_ in kw.items() if k in ("tpp",)})
    return p, ref, gpu, rc


@pytest.mark.parametrize("pot,dims,N", CASES)
def test_pair_sets_bit_exact(simlib, oracle, pot, dims, N):
    p, r, v, D, rc = make_case(pot, dims, oracle.NEWTONIAN, N, seed=1)
    ref = oracle.OracleSystem(p, r, D, force_cutoff=rc)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, force_cutoff=rc, full_list=True)
    gpu.rebuild()
    assert np.array_equal(gpu.pairs(0), ref.half_pairs())
    assert np.array_equal(gpu.pairs(1), ref.full_pairs())
    assert gpu.stats().rebuilds == 1


@pytest.mark.parametrize("pot,dims,N", CASES)
@pytest.mark.parametrize("dyn", [0, 1, 2])
def test_forces_match(simlib, oracle, pot, dims, N, dyn):
    p, r, v, D, rc = make_case(pot, dims, dyn, N, seed=2)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    noise = np.random.default_rng(5).standard_normal((N, dims))
    Fr = ref.calculate_new_forces(noise).copy()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    gpu.rebuild()
    Fg = gpu.forces(noise)
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()


@pytest.mark.parametrize("pot,dims,N", CASES)
def test_energy_virial_match(simlib, oracle, pot, dims, N):
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=3)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    gpu.rebuild()
    e, w, k = gpu.energy()
    assert e == pytest.approx(ref.full_energy(), rel=1e-12)
    assert w == pytest.approx(ref.virial(), rel=1e-12)
    assert k == pytest.approx(ref.kinetic_energy(), rel=1e-12)
    epp = gpu.per_particle_energy()
    assert np.abs(epp - ref.per_particle_energy()).max() <= 1e-12 * np.abs(epp).max()


@pytest.mark.parametrize("pot,dims,N", CASES)
@pytest.mark.parametrize("dyn", [0, 1, 2])
def test_trajectory_with_host_noise(simlib, oracle, pot, dims, N, dyn):
    nsteps = 30
    dt = 2e-5 if dyn == 2 else 0.005  # Brownian from MC-at-kBT=10 starts needs a small step
    p, r, v, D, rc = make_case(pot, dims, dyn, N, seed=4, dt=dt)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    gpu.rebuild()
    noise = np.random.default_rng(6).standard_normal((nsteps, N, dims))
    # first step from the stale F = 0, as the reference
    ref.run(nsteps, noise=noise)
    gpu.step(nsteps, noise=noise)
    rg, vg, Fg, ug = gpu.state()
    L = p.box_size
    assert np.abs(wrap_diff(rg, ref.r, L)).max() < 1e-11
    if dyn != 2:
        assert np.abs(vg - ref.v).max() < 1e-11 * max(1.0, np.abs(ref.v).max())
    assert np.abs(Fg - ref.F).max() < 1e-9 * np.abs(ref.F).max()
    assert np.abs(ug - ref.disp).max() < 1e-11
    assert gpu.stats().rebuilds == ref.rebuilds


@pytest.mark.parametrize("dyn", [1, 2])
def test_philox_noise_matches_oracle_generator(simlib, oracle, dyn):
    N, dims = 1728, 3
    p, r, v, D, rc = make_case(1, dims, dyn, N, seed=8)
    seed = 987654321
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc, seed=seed)
    gpu.rebuild()
    Fg = gpu.forces(None)  # draws Philox step 0
    Fr = ref.calculate_new_forces(oracle.philox_normals(seed, 0, N, dims)).copy()
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()
    assert gpu.stats().noise_draws == 1


def test_many_steps_graph_path_matches_direct(simlib, oracle):
    """The CUDA-graph step loop gives bit-identical results to direct launches."""
    p, r, v, D, rc = make_case(1, 3, 1, 1728, seed=9)
    a = GpuSystem(p, r, D, v=v, force_cutoff=rc, graphs=True)
    b = GpuSystem(p, r, D, v=v, force_cutoff=rc, graphs=False)
    a.rebuild()
    b.rebuild()
    a.step(40)
    b.step(40)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("tpp", [2, 4, 8])
def test_threads_per_particle_same_forces(simlib, oracle, tpp):
    p, r, v, D, rc = make_case(1, 3, 0, 1728, seed=10)
    ref = oracle.OracleSystem(p, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    Fr = ref.calculate_new_forces().copy()
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc, tpp=tpp)
    gpu.rebuild()
    Fg = gpu.forces()
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()


@pytest.mark.parametrize("pot,dims,N", CASES)
def test_split_precision_force_error(simlib, oracle, pot, dims, N):
    from simulationcode_gb300 import _lib
    p, r, v, D, rc = make_case(pot, dims, 0, N, seed=11)
    g64 = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    g32 = GpuSystem(p, r, D, v=v, force_cutoff=rc, precision=_lib.FP32_SPLIT)
    g64.rebuild()
    g32.rebuild()
    F64, F32 = g64.forces(), g32.forces()
    rms = np.sqrt(((F32 - F64) ** 2).sum() / (F64 ** 2).sum())
    assert rms <= 1e-5
    e64, w64, _ = g64.energy()
    e32, w32, _ = g32.energy()
    assert abs(e32 - e64) / N < 1e-5


def test_set_skin_rebuilds_with_new_pair_set(simlib, oracle):
    """simmd_set_skin (the autotuner's rebuild-cadence knob): the lists after
    the change are the reference's lists for the new skin."""
    import ctypes as C
    p, r, v, D, rc = make_case(1, 3, 0, 1728, seed=12)
    gpu = GpuSystem(p, r, D, v=v, force_cutoff=rc)
    gpu.rebuild()
    assert gpu.lib.simmd_set_skin(gpu.ctx, -1, C.c_double(0.5)) == 0
    gpu.rebuild()
    q = oracle.OrcParams.from_buffer_copy(p)
    q.skin = 0.5
    ref = oracle.OracleSystem(q, r, D, v=v, force_cutoff=rc)
    ref.update_neighbor_lists()
    assert np.array_equal(gpu.pairs(0), ref.half_pairs())
    Fr = ref.calculate_new_forces().copy()
    Fg = gpu.forces()
    assert np.abs(Fg - Fr).max() <= 1e-12 * np.abs(Fr).max()


def test_conditional_rebuild_bodies_counted(simlib, oracle):
    """In a captured step loop a rebuild sequence's body runs only when a
    trigger fired: with one replica, bodies run == the replica's rebuilds,
    the kernels counted as run are three a step (kick1+drift, plan, force),
    seven per body run and the closing COM/rescale pass, and the trajectory
    equals direct launches bit for bit."""
    import ctypes as C
    p, r, v, D, rc = make_case(0, 3, 0, 1000, seed=12)
    a = GpuSystem(p, r, D, v=v, force_cutoff=rc, graphs=True)
    b = GpuSystem(p, r, D, v=v, force_cutoff=rc, graphs=False)
    f, rb = C.c_int64(), C.c_int64()
    for g in (a, b):
        g.rebuild()
    assert simlib.simmd_kernel_counts(a.ctx, C.byref(f), C.byref(rb)) == 0
    rb0, l0 = rb.value, simlib.simmd_launch_count(a.ctx)
    for g in (a, b):
        g.step(96)
    assert simlib.simmd_kernel_counts(a.ctx, C.byref(f), C.byref(rb)) == 0
    assert rb.value == a.stats().rebuilds
    assert 1 < a.stats().rebuilds < 96
    assert simlib.simmd_launch_count(a.ctx) - l0 == 3 * 96 + 7 * (rb.value - rb0) + 1
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


def test_split_conversions_match_hardware(simlib):
    """The split-precision kernels widen FP32 to FP64 and round FP64 to FP32
    with integer bit operations (GB300 runs FP64 conversions on its narrow
    FP64 pipe): bit-identical to the hardware converter on 2^24 hashed
    patterns, rounding ties and carries included."""
    import ctypes as C
    bad = C.c_int64(-1)
    for seed in (1, 2):
        assert simlib.simmd_check_conversions(1 << 24, seed, C.byref(bad)) == 0
        assert bad.value == 0
