"""ctypes binding of the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  Arrays follow the reference's ArrayStruct
layout: AoS ``(N, dims)`` float64 (Julia's ``reinterpret(reshape, Float64,
r_array)`` read column-major is the same bytes).  Lists are column-major
``(maxK, N)`` int64 with 0-based ids.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import build as _build

POT_LJ, POT_BERTHIER = 0, 1
NEWTONIAN, LANGEVIN, BROWNIAN = 0, 1, 2


class OrcParams(C.Structure):
    _fields_ = [
        ("dims", C.c_int32), ("potential", C.c_int32), ("dynamics", C.c_int32),
        ("rescale_temperature", C.c_int32), ("N", C.c_int64),
        ("box_size", C.c_double), ("force_cutoff2", C.c_double), ("skin", C.c_double),
        ("lj_eps", C.c_double), ("lj_sigma", C.c_double), ("lj_rc", C.c_double), ("lj_Uc", C.c_double),
        ("b_c0", C.c_double), ("b_c2", C.c_double), ("b_c4", C.c_double), ("b_zeta", C.c_double),
        ("kBT", C.c_double), ("gamma", C.c_double), ("dt", C.c_double), ("m", C.c_double),
    ]


_P_I64 = C.POINTER(C.c_int64)
_P_D = C.POINTER(C.c_double)


class OrcNlist(C.Structure):
    _fields_ = [
        ("maxK", C.c_int64), ("nn_full", _P_I64), ("nn_half", _P_I64),
        ("list_full", _P_I64), ("list_half", _P_I64), ("disp", _P_D), ("disp2", _P_D),
        ("verlet_sphere_size", C.c_double), ("rebuilds", C.c_int64),
        ("overflow", C.c_int32), ("use_cells", C.c_int32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build_oracle()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.orc_berthier_constants.argtypes = [C.c_int64, C.c_double, _P_D, _P_D, _P_D]
        L.orc_lj_Uc.restype = C.c_double
        L.orc_lj_Uc.argtypes = [C.c_double] * 3
        L.orc_verlet_sphere_size.restype = C.c_double
        L.orc_verlet_sphere_size.argtypes = [C.c_double, C.c_double, vp, C.c_int64]
        L.orc_find_mean_D.restype = C.c_double
        L.orc_find_mean_D.argtypes = [vp, C.c_double, C.c_double]
        for fn in ("orc_pair_potential", "orc_pair_force"):
            getattr(L, fn).restype = C.c_double
            getattr(L, fn).argtypes = [vp, C.c_double, C.c_double]
        L.orc_update_neighbor_lists.argtypes = [vp, vp, vp, vp]
        L.orc_calculate_new_forces.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.orc_pair_forces_only.argtypes = [vp, vp, vp, vp, vp]
        for fn in ("orc_calculate_full_energy", "orc_virial"):
            getattr(L, fn).restype = C.c_double
            getattr(L, fn).argtypes = [vp, vp, vp, vp]
        L.orc_compute_potential_energy.argtypes = [vp, vp, vp, vp, vp]
        L.orc_energy_no_neigh.restype = C.c_double
        L.orc_energy_no_neigh.argtypes = [vp, vp, vp]
        L.orc_kinetic_energy.restype = C.c_double
        L.orc_kinetic_energy.argtypes = [vp, vp]
        L.orc_rescale_velocities.argtypes = [vp, vp]
        L.orc_do_time_step.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.orc_run_steps.argtypes = [vp, vp, vp, vp, vp, vp, C.c_int64, vp, C.c_uint64, C.c_uint64]
        L.orc_philox4x32_10.argtypes = [vp, vp, vp]
        L.orc_philox_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, C.c_int32, vp]
        L.orc_generate_diameters_berthier.argtypes = [C.c_int64, C.c_double, C.c_uint64, vp]
        L.orc_random_initial_configuration.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_double,
                                                       C.c_uint64, _P_D]
        L.orc_find_inherent_structure.argtypes = [vp, vp, vp, vp, vp, vp, C.c_double, C.c_int64,
                                                  C.c_double, C.c_double, _P_I64]
        L.orc_relax_capped.argtypes = [vp, vp, vp, vp, vp, C.c_int64, C.c_double, C.c_double]
        L.orc_mc_uniforms.argtypes = [C.c_uint64, C.c_uint64, C.c_int64, vp]
        L.orc_mc_sweeps.argtypes = [vp, vp, vp, vp, C.c_int64, C.c_double, C.c_double, C.c_uint64, C.c_uint64,
                                    vp, _P_D]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def berthier_constants(n=12, rc=1.25):
    c0, c2, c4 = C.c_double(), C.c_double(), C.c_double()
    lib().orc_berthier_constants(n, rc, C.byref(c0), C.byref(c2), C.byref(c4))
    return c0.value, c2.value, c4.value


def make_params(dims, potential, dynamics, N, box_size, force_cutoff2, skin, *, eps=1.0,
                sigma=1.0, lj_rc=2.5, zeta=0.2, berthier_rc=1.25, kBT=0.1, gamma=1.0,
                dt=0.005, m=1.0, rescale=False):
    p = OrcParams()
    p.dims, p.potential, p.dynamics = dims, potential, dynamics
    p.rescale_temperature = int(bool(rescale))
    p.N, p.box_size, p.force_cutoff2, p.skin = N, box_size, force_cutoff2, skin
    p.lj_eps, p.lj_sigma, p.lj_rc = eps, sigma, lj_rc
    p.lj_Uc = lib().orc_lj_Uc(eps, sigma, lj_rc)
    p.b_c0, p.b_c2, p.b_c4 = berthier_constants(12, berthier_rc)
    p.b_zeta = zeta
    p.kBT, p.gamma, p.dt, p.m = kBT, gamma, dt, m
    return p


class OracleSystem:
    """One system's state in the reference layout plus its neighbor lists."""

    def __init__(self, params: OrcParams, r, D, v=None, F=None, maxK=200, force_cutoff=None,
                 use_cells=True):
        self.p = params
        N, d = params.N, params.dims
        self.r = np.ascontiguousarray(np.array(r, dtype=np.float64).reshape(N, d))
        self.D = np.ascontiguousarray(np.array(D, dtype=np.float64).reshape(N))
        self.v = np.zeros((N, d)) if v is None else np.ascontiguousarray(np.array(v, np.float64).reshape(N, d))
        self.F = np.zeros((N, d)) if F is None else np.ascontiguousarray(np.array(F, np.float64).reshape(N, d))
        self.maxK = int(maxK)
        self.nn_full = np.zeros(N, np.int64)
        self.nn_half = np.zeros(N, np.int64)
        self.list_full = np.zeros((N, self.maxK), np.int64)   # row i = column i of the Julia array
        self.list_half = np.zeros((N, self.maxK), np.int64)
        self.disp = np.zeros((N, d))
        self.disp2 = np.zeros(N)
        if force_cutoff is None:
            force_cutoff = math.sqrt(params.force_cutoff2)
        nl = OrcNlist()
        nl.maxK = self.maxK
        nl.nn_full = self.nn_full.ctypes.data_as(_P_I64)
        nl.nn_half = self.nn_half.ctypes.data_as(_P_I64)
        nl.list_full = self.list_full.ctypes.data_as(_P_I64)
        nl.list_half = self.list_half.ctypes.data_as(_P_I64)
        nl.disp = self.disp.ctypes.data_as(_P_D)
        nl.disp2 = self.disp2.ctypes.data_as(_P_D)
        nl.verlet_sphere_size = lib().orc_verlet_sphere_size(params.skin, force_cutoff,
                                                             _ptr(self.D), N)
        nl.rebuilds = 0
        nl.overflow = 0
        nl.use_cells = int(bool(use_cells))
        self.nl = nl

    @property
    def rebuilds(self):
        return self.nl.rebuilds

    def update_neighbor_lists(self):
        st = lib().orc_update_neighbor_lists(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl))
        if st:
            raise RuntimeError("oracle neighbor list overflow (maxK=%d)" % self.maxK)

    def calculate_new_forces(self, noise=None):
        lib().orc_calculate_new_forces(C.byref(self.p), _ptr(self.r), _ptr(self.v), _ptr(self.D),
                                       C.byref(self.nl), _ptr(noise), _ptr(self.F))
        return self.F

    def pair_forces(self):
        F = np.zeros_like(self.r)
        lib().orc_pair_forces_only(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl), _ptr(F))
        return F

    def full_energy(self):
        return lib().orc_calculate_full_energy(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl))

    def per_particle_energy(self):
        e = np.zeros(self.p.N)
        lib().orc_compute_potential_energy(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl), _ptr(e))
        return e

    def energy_no_neigh(self):
        return lib().orc_energy_no_neigh(C.byref(self.p), _ptr(self.r), _ptr(self.D))

    def kinetic_energy(self):
        return lib().orc_kinetic_energy(C.byref(self.p), _ptr(self.v))

    def virial(self):
        return lib().orc_virial(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl))

    def step(self, noise=None):
        st = lib().orc_do_time_step(C.byref(self.p), _ptr(self.r), _ptr(self.v), _ptr(self.F), _ptr(self.D),
                                    C.byref(self.nl), _ptr(noise))
        if st:
            raise RuntimeError("oracle neighbor list overflow")

    def run(self, nsteps, noise=None, seed=0, step0=0):
        if noise is not None:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
        st = lib().orc_run_steps(C.byref(self.p), _ptr(self.r), _ptr(self.v), _ptr(self.F), _ptr(self.D),
                                 C.byref(self.nl), int(nsteps), _ptr(noise), int(seed), int(step0))
        if st:
            raise RuntimeError("oracle neighbor list overflow")

    def relax_capped(self, steps, step_size=1e-3, max_disp=0.05):
        """set-up only: capped steepest descent of the positions"""
        st = lib().orc_relax_capped(C.byref(self.p), _ptr(self.r), _ptr(self.F), _ptr(self.D), C.byref(self.nl),
                                    int(steps), float(step_size), float(max_disp))
        if st:
            raise RuntimeError("oracle neighbor list overflow")

    def mc_sweeps(self, nsweeps, max_disp, swap_prob, seed, sweep0=0):
        """nsweeps of do_MC_step! (translation and swap moves, Philox-keyed
        draws); returns (counts [translations accepted, tried, swaps
        accepted, tried], sum of accepted dE).  Uses the full list."""
        counts = np.zeros(4, np.int64)
        de = C.c_double(0.0)
        st = lib().orc_mc_sweeps(C.byref(self.p), _ptr(self.r), _ptr(self.D), C.byref(self.nl), int(nsweeps),
                                 float(max_disp), float(swap_prob), int(seed), int(sweep0), _ptr(counts),
                                 C.byref(de))
        if st:
            raise RuntimeError("oracle neighbor list overflow")
        return counts, de.value

    def half_pairs(self):
        """Unordered pair set of the half (force) list as a sorted (P,2) int64 array."""
        return _pairs(self.nn_half, self.list_half)

    def full_pairs(self):
        """Unordered pair set of the full (Verlet-sphere) list."""
        return _pairs(self.nn_full, self.list_full, both=True)


def _pairs(nn, lst, both=False):
    N = nn.shape[0]
    rows = np.repeat(np.arange(N, dtype=np.int64), nn)
    mask = np.arange(lst.shape[1])[None, :] < nn[:, None]
    cols = lst[mask]
    a, b = np.minimum(rows, cols), np.maximum(rows, cols)
    pr = np.unique(np.stack([a, b], 1), axis=0) if both else np.stack([a, b], 1)
    order = np.lexsort((pr[:, 1], pr[:, 0]))
    return pr[order]


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


def mc_uniforms(seed, sweep, i):
    out = np.zeros(6)
    lib().orc_mc_uniforms(int(seed), int(sweep), int(i), _ptr(out))
    return out


def philox_normals(seed, step, N, dims):
    out = np.zeros((N, dims))
    lib().orc_philox_normals(int(seed), int(step), int(N), int(dims), _ptr(out))
    return out


def generate_diameters_berthier(N, sigma_ratio=2.219, seed=1):
    D = np.zeros(N)
    lib().orc_generate_diameters_berthier(int(N), float(sigma_ratio), int(seed), _ptr(D))
    return D


def random_initial_configuration(params, D, steps, max_disp=0.1, seed=1, maxK=200, skin=None):
    """MC-relaxed random positions (find_random_initial_configuration!)."""
    N, d = params.N, params.dims
    p = OrcParams.from_buffer_copy(params)
    if skin is not None:
        p.skin = skin
    r = np.zeros((N, d))
    sysm = OracleSystem(p, r, D, maxK=maxK)
    e = C.c_double()
    st = lib().orc_random_initial_configuration(C.byref(p), _ptr(sysm.r), _ptr(sysm.D), C.byref(sysm.nl),
                                                int(steps), float(max_disp), int(seed), C.byref(e))
    if st:
        raise RuntimeError("oracle neighbor list overflow during MC relaxation")
    return sysm.r.copy(), e.value


def find_inherent_structure(sysm: OracleSystem, tolerance=1e-6, max_iterations=10**6,
                            max_step_size=0.001, dt=0.005):
    it = C.c_int64()
    st = lib().orc_find_inherent_structure(C.byref(sysm.p), _ptr(sysm.r), _ptr(sysm.v), _ptr(sysm.F),
                                           _ptr(sysm.D), C.byref(sysm.nl), float(tolerance),
                                           int(max_iterations), float(max_step_size), float(dt),
                                           C.byref(it))
    return st, it.value
