"""Single-replica GPU system driven through the C ABI (ctypes), built from the
same oracle parameters as the CPU reference run."""
from __future__ import annotations

import ctypes as C

import numpy as np

from simulationcode_gb300 import _lib


def to_simmd(op, *, precision=_lib.FP64, force_cutoff, seed=1, max_neighbors=200):
    p = _lib.Params()
    p.dims, p.potential, p.dynamics = op.dims, op.potential, op.dynamics
    p.precision = precision
    p.N = op.N
    p.box_size, p.force_cutoff2, p.skin = op.box_size, op.force_cutoff2, op.skin
    p.verlet_force_cutoff = force_cutoff
    p.lj_eps, p.lj_sigma, p.lj_Uc = op.lj_eps, op.lj_sigma, op.lj_Uc
    p.b_c0, p.b_c2, p.b_c4, p.b_zeta = op.b_c0, op.b_c2, op.b_c4, op.b_zeta
    p.kBT, p.gamma, p.dt, p.m = op.kBT, op.gamma, op.dt, op.m
    p.rescale_temperature = op.rescale_temperature
    p.max_neighbors = max_neighbors
    p.seed = seed
    return p


class GpuSystem:
    def __init__(self, op, r, D, v=None, F=None, *, force_cutoff, precision=_lib.FP64, seed=1, full_list=False,
                 max_neighbors=200, tpp=1, graphs=True):
        self.lib = _lib.load()
        self.N, self.dims = op.N, op.dims
        self.p = to_simmd(op, precision=precision, force_cutoff=force_cutoff, seed=seed,
                          max_neighbors=max_neighbors)
        self.ctx = C.c_void_p()
        _lib.check(self.lib.simmd_create(C.byref(self.p), C.byref(self.ctx)))
        _lib.check(self.lib.simmd_set_tuning(self.ctx, tpp, 1 if graphs else 0, 8))
        if full_list:
            _lib.check(self.lib.simmd_set_full_list(self.ctx, 1))
        r = _lib.f64(r, (self.N, self.dims))
        D = _lib.f64(D, (self.N,))
        v = _lib.f64(v, (self.N, self.dims)) if v is not None else None
        F = _lib.f64(F, (self.N, self.dims)) if F is not None else None
        _lib.check(self.lib.simmd_upload(self.ctx, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), _lib.ptr(D), None))

    def close(self):
        if self.ctx:
            self.lib.simmd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()

    def rebuild(self):
        _lib.check(self.lib.simmd_rebuild(self.ctx))

    def forces(self, noise=None):
        F = np.zeros((self.N, self.dims))
        nz = _lib.f64(noise, (self.N, self.dims)) if noise is not None else None
        _lib.check(self.lib.simmd_forces(self.ctx, _lib.ptr(nz), _lib.ptr(F)))
        return F

    def step(self, nsteps=1, noise=None):
        nz = _lib.f64(noise, (nsteps, self.N, self.dims)) if noise is not None else None
        _lib.check(self.lib.simmd_step(self.ctx, int(nsteps), _lib.ptr(nz)))

    def state(self):
        r = np.zeros((self.N, self.dims))
        v = np.zeros((self.N, self.dims))
        F = np.zeros((self.N, self.dims))
        u = np.zeros((self.N, self.dims))
        _lib.check(self.lib.simmd_download(self.ctx, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), _lib.ptr(u)))
        return r, v, F, u

    def energy(self):
        e, w, k = C.c_double(), C.c_double(), C.c_double()
        _lib.check(self.lib.simmd_energy(self.ctx, C.byref(e), C.byref(w), C.byref(k)))
        return e.value, w.value, k.value

    def per_particle_energy(self):
        e = np.zeros(self.N)
        _lib.check(self.lib.simmd_potential_energy_array(self.ctx, _lib.ptr(e)))
        return e

    def stats(self):
        st = _lib.Stats()
        _lib.check(self.lib.simmd_stats_get(self.ctx, C.byref(st)))
        return st

    def pairs(self, which=0, maxK=200):
        counts = np.zeros(self.N, np.int64)
        lst = np.zeros((self.N, maxK), np.int64)
        _lib.check(self.lib.simmd_export_pairs(self.ctx, which, maxK, _lib.ptr(counts), _lib.ptr(lst)))
        rows = np.repeat(np.arange(self.N, dtype=np.int64), counts)
        mask = np.arange(maxK)[None, :] < counts[:, None]
        cols = lst[mask] - 1
        a, b = np.minimum(rows, cols), np.maximum(rows, cols)
        pr = np.stack([a, b], 1)
        if which == 1:
            pr = np.unique(pr, axis=0)
        return pr[np.lexsort((pr[:, 1], pr[:, 0]))]


def wrap_diff(a, b, L):
    d = a - b
    return d - np.round(d / L) * L
