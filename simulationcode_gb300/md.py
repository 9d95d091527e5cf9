"""Host mirror of SimulationCode.jl's MD interface on top of libsimmd.

Function names follow the reference (Julia's trailing ``!`` becomes a
trailing ``_``); arguments and error behaviour are the same, so a script
written against the reference reads the same here.  Every computation runs in
the CUDA kernels of libsimmd through its C ABI (``_lib``); the host arrays of
``ArrayStruct`` are kept in sync at each call boundary.

Reference map (SimulationCode.jl):
  initialize_neighbor_struct   src/DataStructs.jl:349-378
  update_neighbor_lists!       src/NeighborLists.jl:24-53
  calculate_new_forces!        src/MD.jl:262-316
  do_time_step                 src/MD.jl:429-471, 499-554
  rescale_velocities!          src/MD.jl:391-402
  run_short_MD_equilibration!  src/MD.jl:579-586
  print_log_data               src/MD.jl:610-650
  perform_molecular_dynamics!  src/MD.jl:680-719
  calculate_full_energy        src/AuxiliaryFunctions.jl:22-34
  find_kinetic_energy          src/AuxiliaryFunctions.jl:57-65
  compute_potential_energy!    src/AuxiliaryFunctions.jl:186-196
  logdata                      src/AuxiliaryFunctions.jl:637-646
  create_when_to_save_array    src/Dump.jl:18-31
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import _lib
from .structs import ArrayStruct, Berthier, Brownian, Langevin, LJ, Newtonian, OutputStruct, ParameterStruct


def make_params(parameters: ParameterStruct, skin: float, force_cutoff: float, *, precision=_lib.FP64,
                max_neighbors=200, seed=None) -> _lib.Params:
    """simmd_params from the reference structs."""
    s, U = parameters.system, parameters.interaction_potential
    p = _lib.Params()
    p.dims = s.dims
    if isinstance(U, LJ):
        p.potential = _lib.POT_LJ
        p.lj_eps, p.lj_sigma, p.lj_Uc = U.eps, U.sigma, U.Uc
    elif isinstance(U, Berthier):
        p.potential = _lib.POT_BERTHIER
        p.b_c0, p.b_c2, p.b_c4, p.b_zeta = U.c0, U.c2, U.c4, U.zeta
    else:
        raise ValueError("potential %r is not on the GPU path" % type(U).__name__)
    if isinstance(s, Newtonian):
        p.dynamics, p.m, p.rescale_temperature = _lib.NEWTONIAN, s.m, int(bool(s.rescale_temperature))
    elif isinstance(s, Langevin):
        p.dynamics, p.m, p.gamma = _lib.LANGEVIN, s.m, s.gamma
    elif isinstance(s, Brownian):
        p.dynamics, p.gamma = _lib.BROWNIAN, s.gamma
    else:
        raise ValueError("unknown system type")
    p.kBT, p.dt = s.kBT, s.dt
    p.precision = precision
    p.N = parameters.N
    p.box_size = parameters.box_size
    p.force_cutoff2 = parameters.force_cutoff2
    p.skin = skin
    p.verlet_force_cutoff = force_cutoff
    p.max_neighbors = max_neighbors
    p.seed = parameters.random_seed if seed is None else seed
    return p


class NeighborListStruct:
    """NeighborListStruct (src/DataStructs.jl:243-257), device-backed.

    Holds the scalars of the reference struct; the lists, displacements and
    cell data live on the GPU in the libsimmd context created on first use.
    ``neighbor_numbers_half`` / ``neighbor_list_half`` etc. export the
    device lists in the reference layout on access."""

    def __init__(self, skin_distance, box_size, force_cutoff, N, D_array, dims, maxneighbours=200,
                 precision=_lib.FP64):
        if dims not in (2, 3):
            raise ValueError("To be implemented")
        self.skin_distance = float(skin_distance)
        self.force_cutoff = float(force_cutoff)
        self.verlet_sphere_size = skin_distance + force_cutoff * float(np.max(D_array))
        self.N_cells = int(math.floor(box_size / self.verlet_sphere_size))
        self.cell_size = box_size / self.N_cells if self.N_cells > 0 else box_size
        self.maxneighbours = int(maxneighbours)
        self.precision = precision
        self.N = int(N)
        self.dims = int(dims)
        self.displacement_array = np.zeros((N, dims))
        self.displacement_squared_array = np.zeros(N)
        self.ctx = None
        self._lib = _lib.load()
        self._rebuilds_seen = 0
        self.keep_full_list = False

    # -- device context ---------------------------------------------------
    def _ensure(self, arrays: ArrayStruct, parameters: ParameterStruct):
        if self.ctx is not None:
            return
        p = make_params(parameters, self.skin_distance, self.force_cutoff, precision=self.precision,
                        max_neighbors=self.maxneighbours)
        ctx = C.c_void_p()
        _lib.check(self._lib.simmd_create(C.byref(p), C.byref(ctx)))
        self.ctx = ctx
        if self.keep_full_list:
            _lib.check(self._lib.simmd_set_full_list(ctx, 1))
        _lib.check(self._lib.simmd_upload(ctx, _lib.ptr(arrays.r_array), _lib.ptr(arrays.v_array),
                                          _lib.ptr(arrays.F_array), _lib.ptr(arrays.D_array),
                                          _lib.ptr(self.displacement_array)))

    def push(self, arrays: ArrayStruct):
        _lib.check(self._lib.simmd_set_state(self.ctx, _lib.ptr(arrays.r_array), _lib.ptr(arrays.v_array),
                                             _lib.ptr(arrays.F_array), _lib.ptr(self.displacement_array)))

    def pull(self, arrays: ArrayStruct):
        _lib.check(self._lib.simmd_download(self.ctx, _lib.ptr(arrays.r_array), _lib.ptr(arrays.v_array),
                                            _lib.ptr(arrays.F_array), _lib.ptr(self.displacement_array)))
        d = self.displacement_array
        self.displacement_squared_array[:] = (d * d).sum(1)

    def stats(self) -> _lib.Stats:
        st = _lib.Stats()
        _lib.check(self._lib.simmd_stats_get(self.ctx, C.byref(st)))
        return st

    def _count_rebuilds(self, output: OutputStruct):
        rb = self.stats().rebuilds
        output.N_neighbor_list_rebuilds += rb - self._rebuilds_seen
        self._rebuilds_seen = rb

    def _export(self, which):
        K = self.maxneighbours
        counts = np.zeros(self.N, np.int64)
        lst = np.zeros((self.N, K), np.int64)  # row i = Julia column i
        _lib.check(self._lib.simmd_export_pairs(self.ctx, which, K, _lib.ptr(counts), _lib.ptr(lst)))
        return counts, lst

    @property
    def neighbor_numbers_half(self):
        return self._export(0)[0]

    @property
    def neighbor_list_half(self):
        return self._export(0)[1].T.copy()

    @property
    def neighbor_numbers_full(self):
        return self._export(1)[0]

    @property
    def neighbor_list_full(self):
        return self._export(1)[1].T.copy()

    def __del__(self):
        if getattr(self, "ctx", None) is not None:
            try:
                self._lib.simmd_destroy(self.ctx)
            except Exception:
                pass
            self.ctx = None


def initialize_neighbor_struct(skin_distance, box_size, force_cutoff, N, D_array, dims, maxneighbours=200,
                               precision=_lib.FP64):
    """initialize_neighbor_struct (src/DataStructs.jl:349-378)."""
    return NeighborListStruct(skin_distance, box_size, force_cutoff, N, D_array, dims, maxneighbours, precision)


def update_neighbor_lists_(arrays, parameters, output, neighborlist: NeighborListStruct):
    """update_neighbor_lists! (src/NeighborLists.jl:24-53)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    _lib.check(neighborlist._lib.simmd_rebuild(neighborlist.ctx))
    neighborlist.pull(arrays)
    neighborlist._count_rebuilds(output)


def calculate_new_forces_(arrays, parameters, neighborlist: NeighborListStruct, noise=None):
    """calculate_new_forces! (src/MD.jl:262-316).  ``noise`` (N, dims): the
    N(0,1) deviates of this call's random force (default: the Philox stream)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    nz = _lib.f64(noise, (parameters.N, parameters.system.dims)) if noise is not None else None
    _lib.check(neighborlist._lib.simmd_forces(neighborlist.ctx, _lib.ptr(nz), _lib.ptr(arrays.F_array)))
    if nz is not None:
        arrays.random_displacement[:] = nz


def do_time_step(arrays, parameters, output, neighborlist: NeighborListStruct, system=None, noise=None,
                 nsteps=1):
    """do_time_step (src/MD.jl:429-471, 499-554); ``nsteps`` > 1 runs that
    many steps in one device call.  ``noise``: (nsteps, N, dims) deviates."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    nz = None
    if noise is not None:
        nz = _lib.f64(noise, (nsteps, parameters.N, parameters.system.dims))
    _lib.check(neighborlist._lib.simmd_step(neighborlist.ctx, int(nsteps), _lib.ptr(nz)))
    neighborlist.pull(arrays)
    neighborlist._count_rebuilds(output)


def find_inherent_structure(arrays, parameters, neighborlist: NeighborListStruct, tolerance=1e-6,
                            max_iterations=10 ** 6, max_step_size=0.001, dt=0.005):
    """find_inherent_structure (src/InherentStructure.jl:5-56): steepest
    descent of the positions to the nearest local minimum on the device.
    Returns the iteration count; raises if max_iterations is reached (the
    reference's intent; its own error path raises a MethodError)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    it = (C.c_int64 * 1)()
    st = neighborlist._lib.simmd_inherent_structure(neighborlist.ctx, float(tolerance), int(max_iterations),
                                                    float(max_step_size), float(dt), it)
    neighborlist.pull(arrays)
    _lib.check(st)
    return int(it[0])


def calculate_full_energy(arrays, parameters, neighborlist: NeighborListStruct):
    """calculate_full_energy (src/AuxiliaryFunctions.jl:22-34)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    e = C.c_double()
    _lib.check(neighborlist._lib.simmd_energy(neighborlist.ctx, C.byref(e), None, None))
    return e.value


def calculate_virial(arrays, parameters, neighborlist: NeighborListStruct):
    """W = sum over pairs of r_ij . F_ij (not in the reference)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    w = C.c_double()
    _lib.check(neighborlist._lib.simmd_energy(neighborlist.ctx, None, C.byref(w), None))
    return w.value


def find_kinetic_energy(arrays, parameters, output):
    """find_kinetic_energy (src/AuxiliaryFunctions.jl:57-65): host O(N) sum."""
    v = arrays.v_array
    output.kinetic_energy = float(((v * v).sum(1)).sum()) * (parameters.system.m / 2.0)


def compute_potential_energy_(arrays, parameters, output, neighborlist: NeighborListStruct):
    """compute_potential_energy! (src/AuxiliaryFunctions.jl:186-196)."""
    neighborlist._ensure(arrays, parameters)
    neighborlist.push(arrays)
    _lib.check(neighborlist._lib.simmd_potential_energy_array(neighborlist.ctx,
                                                              _lib.ptr(arrays.potential_energy_array)))


def rescale_velocities_(v_array, parameters):
    """rescale_velocities! (src/MD.jl:391-402)."""
    dims = parameters.system.dims
    ekin = float((v_array * v_array).sum()) * (parameters.system.m / 2.0)
    kbt = 2 * ekin / (dims * parameters.N)
    v_array *= math.sqrt(parameters.system.kBT / kbt)


def run_short_MD_equilibration_(arrays, parameters, output, neighborlist):
    """run_short_MD_equilibration! (src/MD.jl:579-586)."""
    update_neighbor_lists_(arrays, parameters, output, neighborlist)
    if parameters.N_MD_equilibration_steps > 0:
        do_time_step(arrays, parameters, output, neighborlist, nsteps=parameters.N_MD_equilibration_steps)


def logdata(t: int) -> bool:
    """logdata (src/AuxiliaryFunctions.jl:637-646)."""
    if t == 0:
        return True
    l10 = math.log10(t)
    return l10 >= 3 and t % (10 ** int(math.floor(l10))) == 0


def create_when_to_save_array(log_factor, N_starts, N_max):
    """create_when_to_save_array (src/Dump.jl:18-31)."""
    start_times = list(range(0, N_max + 1, max(N_max // N_starts, 1)))
    when = list(start_times)
    for s in start_times:
        t = 1
        while t <= N_max:
            when.append(t + s)
            t = int(math.ceil(t * log_factor))
    when.append(N_max)
    return sorted(set(w for w in when if w <= N_max))


def save_data(arrays, parameters, output, neighborlist, restarted):
    """save_data (src/Dump.jl:60-88): at dump steps rebuild the lists (when not
    restarted, as the reference does) and hand the arrays to the writer."""
    di = parameters.dump_info
    if di is None or not di.save or output.steps_done not in set(di.when_to_save_array):
        return
    if not restarted:
        update_neighbor_lists_(arrays, parameters, output, neighborlist)
    out = {}
    if di.save_r:
        out["positions"] = arrays.r_array.copy()
    if di.save_v:
        out["velocities"] = arrays.v_array.copy()
    if di.save_F:
        out["forces"] = arrays.F_array.copy()
    if di.save_D:
        out["diameters"] = arrays.D_array.copy()
    if di.save_Epot:
        compute_potential_energy_(arrays, parameters, output, neighborlist)
        out["potential_energy"] = arrays.potential_energy_array.copy()
    if di.writer is not None:
        di.writer(output.steps_done, out)


def print_log_data(arrays, parameters, output, neighborlist, start_time):
    """print_log_data (src/MD.jl:610-650) without q4/q6/F2s (out of scope)."""
    output.potential_energy = calculate_full_energy(arrays, parameters, neighborlist)
    if isinstance(parameters.system, Brownian):
        output.kinetic_energy = 0.0
    else:
        find_kinetic_energy(arrays, parameters, output)
    el = time.time() - start_time
    eta = el / max(output.steps_done, 1) * (parameters.N_steps - output.steps_done)
    print("%d/%d, ETA = %.1f, E = %.2f,  E_pot = %.12f,  E_kin = %.2f, kT = %.3f" % (
        output.steps_done, parameters.N_steps, eta, output.potential_energy + output.kinetic_energy,
        output.potential_energy, output.kinetic_energy,
        output.kinetic_energy * 2 / parameters.system.dims / parameters.N), flush=True)


def perform_molecular_dynamics_(arrays, parameters, output, neighborlist, restarted=False,
                                equilibrate_velocities=True, new_file=True, log=True, rng=None):
    """perform_molecular_dynamics! (src/MD.jl:680-719).

    Steps between host-visible events (callback, dump steps, log steps) run
    in one device call; with ``callback=None`` (the reference's no-op
    ``cb(x...) = nothing``) only dump and log steps synchronise."""
    arrays.r_old_array[:] = arrays.r_array
    sysm = parameters.system
    if not restarted and equilibrate_velocities and not isinstance(sysm, Brownian):
        rng = rng if rng is not None else np.random.default_rng(parameters.random_seed)
        arrays.v_array[:] = rng.standard_normal(arrays.v_array.shape) * math.sqrt(sysm.kBT / sysm.m)
    if not restarted:
        output.steps_done = 0
    update_neighbor_lists_(arrays, parameters, output, neighborlist)
    if equilibrate_velocities:
        run_short_MD_equilibration_(arrays, parameters, output, neighborlist)
        if not isinstance(sysm, Brownian):
            rescale_velocities_(arrays.v_array, parameters)
    output.potential_energy = calculate_full_energy(arrays, parameters, neighborlist)
    output.N_neighbor_list_rebuilds = 0
    if new_file:
        save_data(arrays, parameters, output, neighborlist, restarted)
    cb = parameters.callback
    if cb is not None:
        cb(arrays, parameters, output, neighborlist)
    di = parameters.dump_info
    dump_steps = set(di.when_to_save_array) if (di is not None and di.save) else set()
    start = time.time()
    while output.steps_done < parameters.N_steps:
        # next host-visible step
        t = output.steps_done + 1
        if cb is None:
            nxt = parameters.N_steps
            for s in dump_steps:
                if t <= s < nxt:
                    nxt = s
            if log:
                k = t
                while k < nxt and not logdata(k):
                    k = _next_log(k, nxt)
                nxt = min(nxt, k)
            n = max(nxt - output.steps_done, 1)
        else:
            n = 1
        do_time_step(arrays, parameters, output, neighborlist, nsteps=n)
        output.steps_done += n
        if cb is not None:
            cb(arrays, parameters, output, neighborlist)
        save_data(arrays, parameters, output, neighborlist, restarted)
        if log and logdata(output.steps_done):
            print_log_data(arrays, parameters, output, neighborlist, start)
    if log:
        print("MD procedure complete")
        print("Number of neighbor lists built = %d" % output.N_neighbor_list_rebuilds)


def _next_log(k, limit):
    """smallest t > k with logdata(t), capped at limit."""
    if k < 1000:
        return min(limit, 1000)
    p = 10 ** int(math.floor(math.log10(k)))
    return min(limit, (k // p + 1) * p)
