"""Seeded synthetic workloads with the shapes, sizes and value distributions of
the reference's MD configurations (no dataset is involved):

  c1  3D LJ (eps = sigma = 1, rc = 2.5), N = 1000, rho = 1 (L = 10), 10^3
      simple-cubic lattice + uniform jitter +-0.05, Gaussian v at kBT = 0.1
      with zero momentum, Newtonian velocity Verlet dt = 0.01, skin 0.3
  c2  3D polydisperse soft spheres (Berthier), N = 32768, rho = 1.02,
      Langevin gamma = 1, kBT = 0.1, dt = 0.005, skin 0.3
  c3  the c2 system at N = 2^20, Newtonian NVE, dt = 0.005
  c4  512 replicas, N log-uniform in [500, 16384], half 2D / half 3D,
      Berthier at rho = 1.02, Brownian mobility 1, kBT = 0.1, dt = 1e-3,
      skin 0.3
  c5  serving requests: N log-uniform in [256, 65536], dims {2, 3},
      potential {LJ, Berthier}, dynamics {Newtonian, Langevin, Brownian},
      kBT = 0.1, steps log-uniform in [10^3, 10^5]; LJ starts on a simple
      lattice with random vacancies, everything is relaxed before serving
Berthier diameters: regular inverse-CDF quantiles of P(D) ~ D^-3 with
sigma_ratio 2.219 (support [0.7253, 1.6095]), shuffled
(generate_diameters!, src/InitialConfiguration.jl:1-11); positions seeded
uniform random, then relaxed on the GPU by simmd_relax (capped steepest
descent) in place of the reference's MC sweeps at kBT = 10.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .batch import ReplicaSpec
from .structs import Berthier, LJ


def berthier_diameters(N, rng, sigma_ratio=2.219):
    A = 1 / 2 + 1 / (sigma_ratio - 1)
    smin = (1 + sigma_ratio) / (2 * sigma_ratio)
    P = np.linspace(1 / (2 * N), 1 - 1 / (2 * N), N)
    return rng.permutation(np.sqrt(1 / (smin ** -2 - 2 * P / A)))


def gaussian_velocities(N, dims, kBT, m, rng):
    v = rng.standard_normal((N, dims)) * math.sqrt(kBT / m)
    return v - v.mean(0)


def berthier_spec(N, dims, dynamics, rng, *, rho=1.02, skin=0.3, kBT=0.1, gamma=1.0, dt=0.005,
                  precision=_lib.FP64, seed=1, max_neighbors=None):
    U = Berthier()
    L = (N / rho) ** (1.0 / dims)
    D = berthier_diameters(N, rng)
    r = rng.uniform(0.0, L, (N, dims))
    v = gaussian_velocities(N, dims, kBT, 1.0, rng) if dynamics != _lib.BROWNIAN else None
    if max_neighbors is None:
        max_neighbors = 96 if dims == 3 else 40
    return ReplicaSpec(dims=dims, potential=_lib.POT_BERTHIER, dynamics=dynamics, N=N, box_size=L,
                       force_cutoff2=U.rc ** 2, skin=skin, verlet_force_cutoff=U.rc, r=r, D=D, v=v,
                       precision=precision, kBT=kBT, gamma=gamma, dt=dt, b_c0=U.c0, b_c2=U.c2, b_c4=U.c4,
                       b_zeta=U.zeta, max_neighbors=max_neighbors, seed=seed)


def lattice_positions(N, dims, L, rng, jitter=0.05):
    """simple (square/cubic) lattice of n = ceil(N^(1/d)) sites per axis with
    spacing L/n, N sites kept (all of them when N = n^d, else a seeded random
    subset), plus uniform jitter +-``jitter``"""
    n = int(round(N ** (1.0 / dims)))
    if n ** dims < N:
        n += 1
    a = L / n
    g = np.stack(np.meshgrid(*([np.arange(n)] * dims), indexing="ij"), -1).reshape(-1, dims)
    if len(g) > N:
        g = g[np.sort(rng.choice(len(g), N, replace=False))]
    return np.mod((g + 0.5) * a + rng.uniform(-jitter, jitter, (N, dims)), L)


def lj_spec(N, dims, dynamics, rng, *, rho=1.0, skin=0.3, kBT=0.1, gamma=1.0, dt=0.01, precision=_lib.FP64,
            seed=1, lattice=True, max_neighbors=None):
    U = LJ(1.0, 1.0, 2.5)
    L = (N / rho) ** (1.0 / dims)
    n = int(round(N ** (1.0 / dims)))
    if lattice:
        r = lattice_positions(N, dims, L, rng)
    else:
        r = rng.uniform(0.0, L, (N, dims))
    v = gaussian_velocities(N, dims, kBT, 1.0, rng) if dynamics != _lib.BROWNIAN else None
    if max_neighbors is None:
        max_neighbors = 128 if dims == 3 else 48
    return ReplicaSpec(dims=dims, potential=_lib.POT_LJ, dynamics=dynamics, N=N, box_size=L, force_cutoff2=6.25,
                       skin=skin, verlet_force_cutoff=2.5, r=r, D=np.ones(N), v=v, precision=precision, kBT=kBT,
                       gamma=gamma, dt=dt, lj_eps=1.0, lj_sigma=1.0, lj_Uc=U.Uc, max_neighbors=max_neighbors,
                       seed=seed)


def c1(precision=_lib.FP64, seed=1):
    rng = np.random.default_rng(seed)
    return [lj_spec(1000, 3, _lib.NEWTONIAN, rng, dt=0.01, precision=precision, seed=seed)]


def c2(precision=_lib.FP64, seed=2):
    rng = np.random.default_rng(seed)
    return [berthier_spec(32768, 3, _lib.LANGEVIN, rng, dt=0.005, precision=precision, seed=seed)]


def c3(precision=_lib.FP64, seed=3):
    rng = np.random.default_rng(seed)
    return [berthier_spec(1 << 20, 3, _lib.NEWTONIAN, rng, dt=0.005, precision=precision, seed=seed)]


def c4_sizes(nrep=512, seed=4, lo=500, hi=16384):
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), nrep))).astype(int)


def c4(precision=_lib.FP32_SPLIT, seed=4, nrep=512, indices=None):
    """the batch of ``nrep`` replicas; ``indices``: only those replicas (each
    replica depends only on (seed, its index), so a subset equals the same
    replicas of the whole batch)"""
    sizes = c4_sizes(nrep, seed)
    specs = []
    for k in (range(nrep) if indices is None else indices):
        rng = np.random.default_rng(seed * 100003 + k)
        dims = 2 if k % 2 == 0 else 3
        specs.append(berthier_spec(int(sizes[k]), dims, _lib.BROWNIAN, rng, dt=1e-3, precision=precision,
                                   seed=seed * 1000 + k))
    return specs


def lpt_partition(work, nparts):
    """longest-processing-time assignment of independent replicas to
    ``nparts`` GPUs: replicas in decreasing order of work (particles x
    steps), each to the GPU with the least work so far (ties: the lower
    GPU index, then the lower replica index); returns one sorted list of
    replica indices per GPU"""
    import heapq
    heap = [(0, g) for g in range(nparts)]
    parts = [[] for _ in range(nparts)]
    for k in sorted(range(len(work)), key=lambda k: (-work[k], k)):
        load, g = heapq.heappop(heap)
        parts[g].append(k)
        heapq.heappush(heap, (load + work[k], g))
    return [sorted(p) for p in parts]


def c5_draw(rng, nmin=256, nmax=65536, smin=10 ** 3, smax=10 ** 5):
    """one serving request's shape: N log-uniform in [256, 65536], dims in
    {2, 3}, potential in {LJ rc = 2.5, polydisperse soft spheres}, dynamics in
    {Newtonian, Langevin gamma = 1, Brownian}, steps log-uniform in
    [10^3, 10^5]"""
    N = int(math.floor(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
    dims = int(rng.integers(2, 4))
    pot = int(rng.integers(0, 2))
    dyn = int(rng.integers(0, 3))
    steps = int(math.floor(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
    return N, dims, pot, dyn, steps


def c5_spec(N, dims, pot, dyn, rng, seed, precision=_lib.FP32_SPLIT):
    """the replica of a serving request, kBT = 0.1; dt 0.005 for MD, 1e-3
    for Brownian soft spheres, 1e-4 for Brownian LJ (the overdamped update
    is stable only for dt * V'' * neighbours below ~2, and LJ at rho = 1 is
    far stiffer than the soft spheres)"""
    if pot == _lib.POT_LJ:
        dt = 1e-4 if dyn == _lib.BROWNIAN else 0.005
        return lj_spec(N, dims, dyn, rng, dt=dt, precision=precision, seed=seed)
    dt = 1e-3 if dyn == _lib.BROWNIAN else 0.005
    return berthier_spec(N, dims, dyn, rng, dt=dt, precision=precision, seed=seed)


def _c5_rng(seed, k):
    return np.random.default_rng(seed * 1000003 + k)


def c5_draws(n, seed=5):
    """the shapes of ``n`` serving requests (cheap: no configurations)"""
    return [c5_draw(_c5_rng(seed, k)) for k in range(n)]


def c5_requests(n, seed=5, precision=_lib.FP32_SPLIT):
    """(spec, steps) of ``n`` serving requests, seeded; request k has the
    shape ``c5_draws(n, seed)[k]``"""
    out = []
    for k in range(n):
        rng = _c5_rng(seed, k)
        N, dims, pot, dyn, steps = c5_draw(rng)
        out.append((c5_spec(N, dims, pot, dyn, rng, seed * 100000 + k, precision), steps))
    return out


def relax_on_device(specs, device=0, steps=300, step_size=1e-3, cap=0.05):
    """set-up: capped steepest descent of every spec's positions in one FP64
    context on the device (r += step_size*F, |dr| <= cap per step); writes
    the relaxed positions back into the specs and returns the context's
    launch and kernel counts"""
    import copy
    from .batch import ReplicaBatch
    b = ReplicaBatch(device, tpp=1, graphs=True, graph_steps=16)
    n = sum(s.N for s in specs)
    b.reserve(n + 128 * len(specs), n // 2 + 64 * len(specs), len(specs) + 1, max(s.max_neighbors for s in specs))
    ids = []
    for s in specs:
        t = copy.copy(s)
        t.precision = _lib.FP64
        ids.append(b.add(t))
    b.rebuild()
    b.relax(steps, step_size, cap)
    fmax = 0.0
    for s, i in zip(specs, ids):
        r, _, F = b.state(i)
        s.r = r
        fmax = max(fmax, float(np.abs(F).max()))
    counts = (b.launches(),) + tuple(b.kernel_counts())
    b.close()
    return fmax, counts


WORKLOADS = {"c1": c1, "c2": c2, "c3": c3, "c4": c4}

DESCRIPTIONS = {
    "c1": "3D LJ N=1000 rho=1 lattice, Newtonian dt=0.01, skin 0.3",
    "c2": "3D polydisperse soft spheres N=32768 rho=1.02, Langevin gamma=1 kBT=0.1 dt=0.005, skin 0.3",
    "c3": "3D polydisperse soft spheres N=1048576 rho=1.02, Newtonian NVE dt=0.005, skin 0.3",
    "c4": "512 replicas, N log-uniform [500,16384], half 2D/half 3D polydisperse soft spheres rho=1.02, "
          "Brownian mu=1 kBT=0.1 dt=1e-3, skin 0.3",
    "c5": "serving: Poisson requests at 0.8 x measured capacity, N log-uniform [256,65536], dims {2,3}, "
          "potential {LJ, polydisperse soft spheres}, dynamics {Newtonian, Langevin, Brownian}, kBT=0.1, "
          "steps log-uniform [1e3,1e5], 150 GB budget, split precision",
}
