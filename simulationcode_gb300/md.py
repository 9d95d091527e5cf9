"""Host mirror of SimulationCode.jl's MD interface on top of libsimmd.

Function names follow the reference (Julia's trailing ``!`` becomes a
trailing ``_``); arguments and error behaviour are the same, so a script
written against the reference reads the same here.  The reference reaches
its hot path through generic functions that dispatch on their arguments'
types; this module keeps that shape: ``update_neighbor_lists_``,
``calculate_new_forces_``, ``do_time_step``, ``run_short_MD_equilibration_``,
``calculate_full_energy``, ``compute_potential_energy_`` and
``calculate_full_energy_no_neigh`` dispatch on the neighbour-list object,
and the driver ``perform_molecular_dynamics_`` is the reference's loop,
unchanged, written against those generic functions.  With the device-backed
``NeighborListStruct`` of this module every computation runs in the CUDA
kernels of libsimmd through its C ABI (``_lib``); any object with the same
methods (a test's CPU oracle, for instance) can take its place.

Step batching: when the callback is the no-op (``callback=None``, the
reference's ``cb(x...) = nothing``), ``do_time_step`` on the device list
records the step instead of running it, and the recorded steps run in one
device call (CUDA-graph step loop, no host round trip per step) at the next
step whose state the host can see: a dump step, a log step, the last step,
or any call that reads the state through the neighbour list.  With any
other callback every step runs and is copied back before the callback.

Reference map (SimulationCode.jl):
  initialize_neighbor_struct     src/DataStructs.jl:349-378
  update_neighbor_lists!         src/NeighborLists.jl:24-53
  calculate_new_forces!          src/MD.jl:262-316
  do_time_step                   src/MD.jl:429-471, 499-554
  rescale_velocities!            src/MD.jl:391-402
  run_short_MD_equilibration!    src/MD.jl:579-586
  print_log_data                 src/MD.jl:610-650
  perform_molecular_dynamics!    src/MD.jl:680-719
  calculate_full_energy          src/AuxiliaryFunctions.jl:22-34
  find_kinetic_energy            src/AuxiliaryFunctions.jl:57-65
  calculate_full_energy_no_neigh src/AuxiliaryFunctions.jl:86-110
  compute_potential_energy!      src/AuxiliaryFunctions.jl:186-196
  logdata                        src/AuxiliaryFunctions.jl:637-646
  create_when_to_save_array      src/Dump.jl:18-31
  save_data                      src/Dump.jl:60-88
  do_MC_step!                    src/MC.jl:139-156 (translation :21-47, swap :67-110)
  perform_swap_monte_carlo!      src/MC.jl:180-243
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


def _dump_step(parameters, step):
    di = parameters.dump_info
    return di is not None and di.save and step in di._when_set()


class NeighborListStruct:
    """NeighborListStruct (src/DataStructs.jl:243-257), device-backed.

    Holds the scalars of the reference struct; the lists, displacements and
    cell data live on the GPU in the libsimmd context created on first use.
    ``neighbor_numbers_half`` / ``neighbor_list_half`` etc. export the
    device lists in the reference layout on access.

    Host/device protocol: the host arrays of ``ArrayStruct`` are pushed to
    the device before each device operation (``simmd_set_state``, lists
    kept) and copied back after it, except while steps are recorded for a
    batched run (``pending``): then the host arrays are those of the last
    copy-back and are neither read nor written until the recorded steps
    run."""

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
        self.pending = 0           # recorded steps not yet run on the device
        self.pending_mc = None     # recorded MC sweeps: [count, max_displacement, swap_probability]
        self.device_calls = 0      # simmd_step / simmd_mc_sweeps calls made (batching evidence)
        self._output = None        # OutputStruct of the recorded steps
        self._mc_seen = (np.zeros(4, np.int64), 0.0)

    # -- device context ---------------------------------------------------
    def _ensure(self, arrays: ArrayStruct, parameters: ParameterStruct):
        if self.ctx is not None:
            return
        p = make_params(parameters, self.skin_distance, self.force_cutoff, precision=self.precision,
                        max_neighbors=self.maxneighbours)
        ctx = C.c_void_p()
        _lib.check(self._lib.simmd_create(C.byref(p), C.byref(ctx)))
        self.ctx = ctx
        self._params = p
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

    def _count_rebuilds(self, output):
        output = output if output is not None else self._output
        rb = self.stats().rebuilds
        if output is not None:
            output.N_neighbor_list_rebuilds += rb - self._rebuilds_seen
        self._rebuilds_seen = rb

    def _begin(self, arrays, parameters, output):
        """before a device operation: create the context, run recorded
        steps or sweeps, push the host arrays"""
        self._ensure(arrays, parameters)
        if self.pending:
            self._run(arrays, output, 0)
        if self.pending_mc is not None:
            self._run_mc(arrays, output, 0, *self.pending_mc[1:])
        self.push(arrays)

    def _run_mc(self, arrays, output, extra, max_disp, swap_prob):
        """run the recorded MC sweeps plus ``extra``, then copy back r, D and
        the move counters"""
        n = (self.pending_mc[0] if self.pending_mc is not None else 0) + extra
        self.pending_mc = None
        if n == 0:
            return
        self.push(arrays)
        _lib.check(self._lib.simmd_mc_sweeps(self.ctx, int(n), float(max_disp), float(swap_prob)))
        self.device_calls += 1
        self.pull(arrays)
        _lib.check(self._lib.simmd_download_diameters(self.ctx, 0, _lib.ptr(arrays.D_array)))
        counts = np.zeros(4, np.int64)
        de = C.c_double()
        _lib.check(self._lib.simmd_mc_stats(self.ctx, 0, _lib.ptr(counts), C.byref(de)))
        c0, d0 = self._mc_seen
        out = output if output is not None else self._output
        if out is not None:
            dc = counts - c0
            out.N_translations_accepted += int(dc[0])
            out.N_translations_total += int(dc[1])
            out.N_swaps_accepted += int(dc[2])
            out.N_swaps_total += int(dc[3])
            out.potential_energy += de.value - d0
        self._mc_seen = (counts, de.value)
        self._count_rebuilds(output)

    def _run(self, arrays, output, extra):
        """run the recorded steps plus ``extra`` from the host state of the
        last copy-back, then copy back"""
        n = self.pending + extra
        self.pending = 0
        if n == 0:
            return
        self.push(arrays)
        _lib.check(self._lib.simmd_step(self.ctx, int(n), None))
        self.device_calls += 1
        self.pull(arrays)
        self._count_rebuilds(output)

    def flush(self, arrays, parameters, output):
        """run the recorded steps or sweeps now (the host arrays become current)"""
        if self.pending:
            self._ensure(arrays, parameters)
            self._run(arrays, output, 0)
        if self.pending_mc is not None:
            self._ensure(arrays, parameters)
            self._run_mc(arrays, output, 0, *self.pending_mc[1:])

    def do_MC_step_(self, arrays, parameters, output, swap_probability):
        """do_MC_step! (src/MC.jl:139-156): one sweep of translation and swap
        moves on the device; with the no-op callback, sweeps are recorded and
        run together at the next sweep whose state the host sees"""
        self._ensure(arrays, parameters)
        if self.pending:
            self._run(arrays, output, 0)
        md_ = float(parameters.max_MC_displacement)
        key = (md_, float(swap_probability))
        if parameters.callback is None:
            after = output.steps_done + 1  # steps_done advances after this call
            self._output = output
            if not (_dump_step(parameters, after) or logdata(after) or after > parameters.N_steps):
                if self.pending_mc is not None and tuple(self.pending_mc[1:]) != key:
                    self._run_mc(arrays, output, 0, *self.pending_mc[1:])
                if self.pending_mc is None:
                    self.pending_mc = [0, md_, float(swap_probability)]
                self.pending_mc[0] += 1
                return
        if self.pending_mc is not None and tuple(self.pending_mc[1:]) != key:
            self._run_mc(arrays, output, 0, *self.pending_mc[1:])
        self._run_mc(arrays, output, 1, *key)

    # -- the reference's hot-path functions, device methods ----------------
    def update_neighbor_lists_(self, arrays, parameters, output):
        self._begin(arrays, parameters, output)
        _lib.check(self._lib.simmd_rebuild(self.ctx))
        self.pull(arrays)
        self._count_rebuilds(output)

    def calculate_new_forces_(self, arrays, parameters, noise=None):
        self._begin(arrays, parameters, None)
        nz = _lib.f64(noise, (parameters.N, parameters.system.dims)) if noise is not None else None
        _lib.check(self._lib.simmd_forces(self.ctx, _lib.ptr(nz), _lib.ptr(arrays.F_array)))
        if nz is not None:
            arrays.random_displacement[:] = nz

    def do_time_step(self, arrays, parameters, output, system, noise=None, nsteps=1):
        self._ensure(arrays, parameters)
        if noise is None and nsteps == 1 and parameters.callback is None:
            # batch: record the step unless the host sees the state after it
            # (output.steps_done is advanced by the driver after this call)
            step = output.steps_done + 1
            self._output = output
            if not (_dump_step(parameters, step) or logdata(step) or step >= parameters.N_steps):
                self.pending += 1
                return
            self._run(arrays, output, 1)
            return
        self._begin(arrays, parameters, output)
        nz = None
        if noise is not None:
            nz = _lib.f64(noise, (nsteps, parameters.N, parameters.system.dims))
        _lib.check(self._lib.simmd_step(self.ctx, int(nsteps), _lib.ptr(nz)))
        self.device_calls += 1
        self.pull(arrays)
        self._count_rebuilds(output)

    def run_short_MD_equilibration_(self, arrays, parameters, output):
        self.update_neighbor_lists_(arrays, parameters, output)
        if parameters.N_MD_equilibration_steps > 0:
            self.do_time_step(arrays, parameters, output, parameters.system,
                              nsteps=parameters.N_MD_equilibration_steps)

    def calculate_full_energy(self, arrays, parameters):
        self._begin(arrays, parameters, None)
        e = C.c_double()
        _lib.check(self._lib.simmd_energy(self.ctx, C.byref(e), None, None))
        return e.value

    def calculate_virial(self, arrays, parameters):
        self._begin(arrays, parameters, None)
        w = C.c_double()
        _lib.check(self._lib.simmd_energy(self.ctx, None, C.byref(w), None))
        return w.value

    def compute_potential_energy_(self, arrays, parameters, output):
        self._begin(arrays, parameters, output)
        _lib.check(self._lib.simmd_potential_energy_array(self.ctx, _lib.ptr(arrays.potential_energy_array)))

    def calculate_full_energy_no_neigh(self, arrays, parameters):
        """the reference's E_pot_test cross-check: the energy of the current
        positions from lists built afresh (a temporary context: cell binning
        and Verlet build of the positions as they are now, then the energy
        pass), independent of the running lists and their skin bookkeeping"""
        self._begin(arrays, parameters, None)
        tmp = C.c_void_p()
        _lib.check(self._lib.simmd_create(C.byref(self._params), C.byref(tmp)))
        try:
            _lib.check(self._lib.simmd_upload(tmp, _lib.ptr(arrays.r_array), None, None, _lib.ptr(arrays.D_array),
                                              None))
            e = C.c_double()
            _lib.check(self._lib.simmd_energy(tmp, C.byref(e), None, None))
        finally:
            self._lib.simmd_destroy(tmp)
        return e.value

    def find_inherent_structure(self, arrays, parameters, tolerance, max_iterations, max_step_size, dt):
        self._begin(arrays, parameters, None)
        it = (C.c_int64 * 1)()
        st = self._lib.simmd_inherent_structure(self.ctx, float(tolerance), int(max_iterations),
                                                float(max_step_size), float(dt), it)
        self.pull(arrays)
        _lib.check(st)
        return int(it[0])

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


# ---------------------------------------------------------------------------
# generic functions: dispatch on the neighbour list, as the reference's
# methods dispatch on their argument types
# ---------------------------------------------------------------------------
def update_neighbor_lists_(arrays, parameters, output, neighborlist):
    """update_neighbor_lists! (src/NeighborLists.jl:24-53)."""
    neighborlist.update_neighbor_lists_(arrays, parameters, output)


def calculate_new_forces_(arrays, parameters, neighborlist, noise=None):
    """calculate_new_forces! (src/MD.jl:262-316).  ``noise`` (N, dims): the
    N(0,1) deviates of this call's random force (default: the Philox stream)."""
    neighborlist.calculate_new_forces_(arrays, parameters, noise)


def do_time_step(arrays, parameters, output, neighborlist, system=None, noise=None, nsteps=1):
    """do_time_step (src/MD.jl:429-471, 499-554); ``nsteps`` > 1 runs that
    many steps in one device call.  ``noise``: (nsteps, N, dims) deviates."""
    neighborlist.do_time_step(arrays, parameters, output, parameters.system if system is None else system,
                              noise=noise, nsteps=nsteps)


def run_short_MD_equilibration_(arrays, parameters, output, neighborlist):
    """run_short_MD_equilibration! (src/MD.jl:579-586)."""
    neighborlist.run_short_MD_equilibration_(arrays, parameters, output)


def calculate_full_energy(arrays, parameters, neighborlist):
    """calculate_full_energy (src/AuxiliaryFunctions.jl:22-34)."""
    return neighborlist.calculate_full_energy(arrays, parameters)


def calculate_virial(arrays, parameters, neighborlist):
    """W = sum over pairs of r_ij . F_ij (not in the reference)."""
    return neighborlist.calculate_virial(arrays, parameters)


def compute_potential_energy_(arrays, parameters, output, neighborlist):
    """compute_potential_energy! (src/AuxiliaryFunctions.jl:186-196)."""
    neighborlist.compute_potential_energy_(arrays, parameters, output)


def calculate_full_energy_no_neigh(arrays, parameters, neighborlist):
    """calculate_full_energy_no_neigh (src/AuxiliaryFunctions.jl:86-110):
    the energy without the running neighbour lists (E_pot_test)."""
    return neighborlist.calculate_full_energy_no_neigh(arrays, parameters)


def find_inherent_structure(arrays, parameters, neighborlist, tolerance=1e-6, max_iterations=10 ** 6,
                            max_step_size=0.001, dt=0.005):
    """find_inherent_structure (src/InherentStructure.jl:5-56): steepest
    descent of the positions to the nearest local minimum on the device.
    Returns the iteration count; raises if max_iterations is reached (the
    reference's intent; its own error path raises a MethodError)."""
    return neighborlist.find_inherent_structure(arrays, parameters, tolerance, max_iterations, max_step_size, dt)


def do_MC_step_(arrays, parameters, output, neighborlist, swap_probability):
    """do_MC_step! (src/MC.jl:139-156): one sweep of Metropolis translation
    and swap moves."""
    neighborlist.do_MC_step_(arrays, parameters, output, swap_probability)


def perform_swap_monte_carlo_(arrays, parameters, output, neighborlist, stepsdone=0, log=print):
    """perform_swap_monte_carlo! (src/MC.jl:180-243), the reference's loop:
    sweeps until steps_done passes N_steps, with the callback, save_data and
    the log line (E_pot kept by adding each accepted move's dE, and
    E_pot_test recomputed without the running lists).  Returns the logged
    values (q4/q6/F2s are out of scope)."""
    say = log if log is not None else (lambda m: None)
    if getattr(neighborlist, "ctx", 0) is None:  # a device list not yet in use: keep the full list from the start
        neighborlist.keep_full_list = True
    update_neighbor_lists_(arrays, parameters, output, neighborlist)
    output.kinetic_energy = calculate_full_energy(arrays, parameters, neighborlist)
    output.steps_done = stepsdone
    output.N_swaps_total = 0
    output.N_swaps_accepted = 0
    output.N_translations_total = 0
    output.N_translations_accepted = 0
    output.N_neighbor_list_rebuilds = 0
    arrays.r_old_array[:] = arrays.r_array
    if stepsdone == 0:
        save_data(arrays, parameters, output, neighborlist, False)
    cb = parameters.callback
    if cb is not None:
        cb(arrays, parameters, output, neighborlist)
    output.potential_energy = calculate_full_energy_no_neigh(arrays, parameters, neighborlist)
    logged = []
    while output.steps_done <= parameters.N_steps:
        do_MC_step_(arrays, parameters, output, neighborlist, parameters.swap_probability)
        if cb is not None:
            cb(arrays, parameters, output, neighborlist)
        output.steps_done += 1
        save_data(arrays, parameters, output, neighborlist, False)
        if logdata(output.steps_done):
            flush = getattr(neighborlist, "flush", None)
            if flush is not None:
                flush(arrays, parameters, output)
            energy_no_neigh = calculate_full_energy_no_neigh(arrays, parameters, neighborlist)
            say("%d/%d, E_pot = %.12f,  E_pot_test = %.12f" % (output.steps_done, parameters.N_steps,
                                                                output.potential_energy, energy_no_neigh))
            logged.append({"step": output.steps_done, "E_pot": output.potential_energy,
                           "E_pot_test": energy_no_neigh})
    flush = getattr(neighborlist, "flush", None)
    if flush is not None:
        flush(arrays, parameters, output)
    say("Completed the MC procedure.")
    say("Number of neighbor lists built = %d" % output.N_neighbor_list_rebuilds)
    say("Swap moves accepted: %d/%d" % (output.N_swaps_accepted, output.N_swaps_total))
    say("Translation moves accepted: %d/%d" % (output.N_translations_accepted, output.N_translations_total))
    return logged


def find_kinetic_energy(arrays, parameters, output):
    """find_kinetic_energy (src/AuxiliaryFunctions.jl:57-65)."""
    v = arrays.v_array
    # the reference's order: per particle sum(v.^2), accumulated in turn
    ekin = float(np.cumsum((v * v).sum(1))[-1])
    output.kinetic_energy = ekin * (parameters.system.m / 2.0)


def rescale_velocities_(v_array, parameters):
    """rescale_velocities! (src/MD.jl:391-402)."""
    dims = parameters.system.dims
    ekin = float(np.cumsum((v_array * v_array).sum(1))[-1])
    ekin *= parameters.system.m / 2.0
    kbt = 2 * ekin / (dims * parameters.N)
    v_array *= math.sqrt(parameters.system.kBT / kbt)


def save_data(arrays, parameters, output, neighborlist, restarted):
    """save_data (src/Dump.jl:60-88): at dump steps rebuild the lists (when not
    restarted, as the reference does) and hand the arrays to the writer (the
    reference writes them to HDF5)."""
    di = parameters.dump_info
    if di is None or not (di.save and output.steps_done in di._when_set()):
        return
    elif not restarted:
        update_neighbor_lists_(arrays, parameters, output, neighborlist)  # for complete reproducibility
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


def print_log_data(arrays, parameters, output, neighborlist, start_time, log=print):
    """print_log_data (src/MD.jl:610-650) without q4/q6/F2s (out of scope),
    with the E_pot_test cross-check.  Returns the logged values."""
    el = time.time() - start_time
    remaining = el / max(output.steps_done, 1) * (parameters.N_steps - output.steps_done)
    output.potential_energy = calculate_full_energy(arrays, parameters, neighborlist)
    if not isinstance(parameters.system, Brownian):
        find_kinetic_energy(arrays, parameters, output)
    else:
        output.kinetic_energy = 0.0
    energy_no_neigh = calculate_full_energy_no_neigh(arrays, parameters, neighborlist)
    if log is not None:
        log("%d/%d, ETA = %.1f, E = %.2f,  E_pot = %.12f,  E_pot_test = %.12f,  E_kin = %.2f, kT = %.3f" % (
            output.steps_done, parameters.N_steps, remaining, output.potential_energy + output.kinetic_energy,
            output.potential_energy, energy_no_neigh, output.kinetic_energy,
            output.kinetic_energy * 2 / parameters.system.dims / parameters.N))
    return {"step": output.steps_done, "E_pot": output.potential_energy, "E_pot_test": energy_no_neigh,
            "E_kin": output.kinetic_energy}


def perform_molecular_dynamics_(arrays, parameters, output, neighborlist, restarted=False,
                                equilibrate_velocities=True, new_file=True, log=print, rng=None):
    """perform_molecular_dynamics! (src/MD.jl:680-719), the reference's loop.

    ``rng`` draws the velocity randomisation (the reference's ``randn!`` on
    the global generator; default: seeded by ``parameters.random_seed``).
    ``log`` receives the printed lines (None: silent).  Returns the list of
    logged values (one dict per log step)."""
    say = log if log is not None else (lambda m: None)
    say("\n\nStarting MD procedure")
    arrays.r_old_array[:] = arrays.r_array
    sysm = parameters.system
    if not restarted and equilibrate_velocities and not isinstance(sysm, Brownian):
        rng = rng if rng is not None else np.random.default_rng(parameters.random_seed)
        arrays.v_array[:] = rng.standard_normal(arrays.v_array.shape)
        arrays.v_array *= math.sqrt(sysm.kBT / sysm.m)
    if not restarted:
        output.steps_done = 0
    say("Running production MD")
    update_neighbor_lists_(arrays, parameters, output, neighborlist)
    if equilibrate_velocities:
        run_short_MD_equilibration_(arrays, parameters, output, neighborlist)
        if not isinstance(sysm, Brownian):  # a Brownian system has no velocities
            rescale_velocities_(arrays.v_array, parameters)
    output.potential_energy = calculate_full_energy(arrays, parameters, neighborlist)
    output.N_neighbor_list_rebuilds = 0
    if new_file:
        save_data(arrays, parameters, output, neighborlist, restarted)
    cb = parameters.callback
    if cb is not None:
        cb(arrays, parameters, output, neighborlist)
    start_time = time.time()
    logged = []
    while output.steps_done < parameters.N_steps:
        do_time_step(arrays, parameters, output, neighborlist, parameters.system)
        output.steps_done += 1
        if cb is not None:
            cb(arrays, parameters, output, neighborlist)
        save_data(arrays, parameters, output, neighborlist, restarted)
        if logdata(output.steps_done):
            logged.append(print_log_data(arrays, parameters, output, neighborlist, start_time, log))
    flush = getattr(neighborlist, "flush", None)
    if flush is not None:  # N_steps <= steps_done on entry leaves nothing recorded; kept for safety
        flush(arrays, parameters, output)
    say("MD procedure complete")
    say("Number of neighbor lists built = %d" % output.N_neighbor_list_rebuilds)
    return logged
