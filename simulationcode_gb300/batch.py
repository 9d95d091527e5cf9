"""Many independent replicas in one libsimmd context (one stream, one slot
space, one CUDA-graph step loop): the batched front end.

Each replica is a full system (its own N, dims, potential, dynamics,
precision, box and seed).  All replicas advance together by ``step``; every
kernel launch covers all of them, and the per-replica results are
bit-identical to running the replica alone (same slot layout inside the
replica, per-replica reductions in a fixed order, noise keyed by the
replica's seed and original particle ids).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional

import numpy as np

from . import _lib


@dataclasses.dataclass
class ReplicaSpec:
    """One replica: the scalars of simmd_params plus its initial arrays."""
    dims: int
    potential: int
    dynamics: int
    N: int
    box_size: float
    force_cutoff2: float
    skin: float
    verlet_force_cutoff: float
    r: np.ndarray
    D: np.ndarray
    v: Optional[np.ndarray] = None
    precision: int = _lib.FP64
    kBT: float = 0.1
    gamma: float = 1.0
    dt: float = 0.005
    m: float = 1.0
    lj_eps: float = 1.0
    lj_sigma: float = 1.0
    lj_Uc: float = 0.0
    b_c0: float = 0.0
    b_c2: float = 0.0
    b_c4: float = 0.0
    b_zeta: float = 0.2
    rescale_temperature: bool = False
    max_neighbors: int = 200
    seed: int = 1

    def params(self) -> _lib.Params:
        p = _lib.Params()
        for f in ("dims", "potential", "dynamics", "precision", "N", "box_size", "force_cutoff2", "skin",
                  "verlet_force_cutoff", "lj_eps", "lj_sigma", "lj_Uc", "b_c0", "b_c2", "b_c4", "b_zeta", "kBT",
                  "gamma", "dt", "m", "max_neighbors", "seed"):
            setattr(p, f, getattr(self, f))
        p.rescale_temperature = int(bool(self.rescale_temperature))
        return p

    def device_bytes(self) -> int:
        """device bytes this replica occupies in a context (admission)"""
        p = self.params()
        return int(_lib.load().simmd_replica_bytes(C.byref(p), self.max_neighbors))


class ReplicaBatch:
    """A libsimmd context holding many replicas."""

    def __init__(self, device: int = 0, *, tpp: int = 1, graphs: bool = True, graph_steps: int = 16):
        self.lib = _lib.load()
        self.ctx = C.c_void_p()
        _lib.check(self.lib.simmd_engine_create(device, C.byref(self.ctx)))
        _lib.check(self.lib.simmd_set_tuning(self.ctx, tpp, int(graphs), graph_steps))
        self.specs = {}
        self.inner_skin = 0.0  # inner skin of the filtered force-pass lists (0: none)

    def reserve(self, slots: int, cells: int, replicas: int, max_neighbors: int = 200):
        _lib.check(self.lib.simmd_reserve(self.ctx, slots, cells, replicas, max_neighbors))

    def add(self, spec: ReplicaSpec) -> int:
        p = spec.params()
        r = _lib.f64(spec.r, (spec.N, spec.dims))
        D = _lib.f64(spec.D, (spec.N,))
        v = _lib.f64(spec.v, (spec.N, spec.dims)) if spec.v is not None else None
        rid = C.c_int32()
        _lib.check(self.lib.simmd_add_replica(self.ctx, C.byref(p), _lib.ptr(r), _lib.ptr(v), None, _lib.ptr(D),
                                              C.byref(rid)))
        self.specs[rid.value] = spec
        return rid.value

    def remove(self, rid: int):
        _lib.check(self.lib.simmd_remove_replica(self.ctx, rid))
        self.specs.pop(rid, None)

    def rebuild(self):
        _lib.check(self.lib.simmd_rebuild(self.ctx))

    def relax(self, nsteps: int, step_size: float = 1e-3, max_disp: float = 0.05):
        """capped steepest descent r += step_size*F, |dr| <= max_disp (set-up)"""
        _lib.check(self.lib.simmd_relax(self.ctx, nsteps, step_size, max_disp))

    def inherent_structure(self, tolerance=1e-6, max_iterations=10 ** 6, max_step_size=0.001, dt=0.005,
                           allow_not_converged=False):
        """minimise every replica (find_inherent_structure); returns
        {replica id: iterations}.  Raises if a replica reached
        max_iterations unless ``allow_not_converged``."""
        n = max(self.specs) + 1 if self.specs else 1
        it = (C.c_int64 * n)()
        st = self.lib.simmd_inherent_structure(self.ctx, float(tolerance), int(max_iterations),
                                               float(max_step_size), float(dt), it)
        if not (allow_not_converged and st == _lib.ERR_NOT_CONVERGED):
            _lib.check(st)
        return {rid: int(it[rid]) for rid in self.specs}

    def step(self, nsteps: int):
        _lib.check(self.lib.simmd_step(self.ctx, int(nsteps), None))

    def step_async_status(self, nsteps: int) -> int:
        """step, returning the status instead of raising (serving loop)."""
        return int(self.lib.simmd_step(self.ctx, int(nsteps), None))

    def transfer_layout(self):
        """batched host layout of upload_all / download_all: (total rows,
        {replica id: first row}) of a (rows, dims_r) stack of every replica's
        (N, dims) block in replica-id order, as flat float64 offsets"""
        n = max(self.specs) + 1 if self.specs else 1
        off = np.full(n, -1, np.int64)
        total = int(self.lib.simmd_transfer_layout(self.ctx, n, _lib.ptr(off)))
        return total, {rid: int(off[rid]) for rid in self.specs}

    def upload_all(self, r: np.ndarray, D: np.ndarray, v: Optional[np.ndarray] = None,
                   F: Optional[np.ndarray] = None):
        """simmd_upload_all: every replica from flat float64 arrays in the
        batched layout (r, v, F: the replicas' (N, dims) blocks in id order;
        D: their N diameters in id order)"""
        _lib.check(self.lib.simmd_upload_all(self.ctx, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), _lib.ptr(D), None))

    def set_state_all(self, r: Optional[np.ndarray] = None, v: Optional[np.ndarray] = None,
                      F: Optional[np.ndarray] = None, disp: Optional[np.ndarray] = None):
        """simmd_set_state_all: every replica's state overwritten in place from
        flat float64 arrays in the batched layout (any may be None), keeping
        the lists and the skin bookkeeping"""
        _lib.check(self.lib.simmd_set_state_all(self.ctx, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), _lib.ptr(disp)))

    def download_all(self, r: Optional[np.ndarray] = None, v: Optional[np.ndarray] = None,
                     F: Optional[np.ndarray] = None):
        """simmd_download_all into flat float64 arrays in the batched layout"""
        _lib.check(self.lib.simmd_download_all(self.ctx, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), None))

    def mc_sweeps(self, nsweeps: int, max_displacement: float, swap_probability: float):
        """swap Monte Carlo: nsweeps of do_MC_step! for every replica (serial
        chain per replica, FP64 find_energy, rebuilds inside sweeps)"""
        _lib.check(self.lib.simmd_mc_sweeps(self.ctx, int(nsweeps), float(max_displacement),
                                            float(swap_probability)))

    def mc_stats(self, rid: int):
        """(counts [translations accepted, tried, swaps accepted, tried],
        sum of accepted dE)"""
        counts = np.zeros(4, np.int64)
        de = C.c_double()
        _lib.check(self.lib.simmd_mc_stats(self.ctx, rid, _lib.ptr(counts), C.byref(de)))
        return counts, de.value

    def diameters(self, rid: int) -> np.ndarray:
        D = np.zeros(self.specs[rid].N)
        _lib.check(self.lib.simmd_download_diameters(self.ctx, rid, _lib.ptr(D)))
        return D

    def state(self, rid: int):
        s = self.specs[rid]
        r = np.zeros((s.N, s.dims))
        v = np.zeros((s.N, s.dims))
        F = np.zeros((s.N, s.dims))
        _lib.check(self.lib.simmd_download_r(self.ctx, rid, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F), None))
        return r, v, F

    def dump_async(self, rid: int, r: np.ndarray, v: Optional[np.ndarray] = None, F: Optional[np.ndarray] = None):
        """queue a copy of the replica's current r (v, F) into the given
        float64 arrays (shape (N, dims), C order; page-locked with
        host_register for the copy to overlap later steps)"""
        s = self.specs[rid]
        for a in (r, v, F):
            if a is not None and (a.dtype != np.float64 or a.shape != (s.N, s.dims) or not a.flags.c_contiguous):
                raise ValueError("dump arrays must be C-contiguous float64 of shape (N, dims)")
        self._dump_refs = (r, v, F)   # keep them alive until the wait
        _lib.check(self.lib.simmd_dump_async(self.ctx, rid, _lib.ptr(r), _lib.ptr(v), _lib.ptr(F)))

    def dump_wait(self):
        _lib.check(self.lib.simmd_dump_wait(self.ctx))
        self._dump_refs = None

    def host_register(self, a: np.ndarray):
        _lib.check(self.lib.simmd_host_register(C.c_void_p(a.ctypes.data), a.nbytes))

    def host_unregister(self, a: np.ndarray):
        _lib.check(self.lib.simmd_host_unregister(C.c_void_p(a.ctypes.data)))

    def energies(self):
        _lib.check(self.lib.simmd_energy_all(self.ctx))
        return {rid: self.stats(rid) for rid in self.specs}

    def stats(self, rid: int) -> _lib.Stats:
        st = _lib.Stats()
        _lib.check(self.lib.simmd_stats_r(self.ctx, rid, C.byref(st)))
        return st

    def launches(self) -> int:
        return int(self.lib.simmd_launch_count(self.ctx))

    def kernel_counts(self):
        f, r = C.c_int64(), C.c_int64()
        _lib.check(self.lib.simmd_kernel_counts(self.ctx, C.byref(f), C.byref(r)))
        return f.value, r.value

    def device_bytes(self) -> int:
        return int(self.lib.simmd_device_bytes(self.ctx))

    def set_budget(self, nbytes: int):
        """cap on the context's capacity grows (0 = none)"""
        _lib.check(self.lib.simmd_set_budget(self.ctx, int(nbytes)))

    def replica_bytes(self, spec: "ReplicaSpec") -> int:
        p = spec.params()
        return int(self.lib.simmd_replica_bytes(C.byref(p), spec.max_neighbors))

    def timer_start(self):
        _lib.check(self.lib.simmd_timer_start(self.ctx))

    def timer_stop(self) -> float:
        ms = C.c_float()
        _lib.check(self.lib.simmd_timer_stop(self.ctx, C.byref(ms)))
        return ms.value

    def profile(self, enable: bool):
        _lib.check(self.lib.simmd_set_profile(self.ctx, int(enable)))

    def profile_get(self):
        out = np.zeros(6)
        _lib.check(self.lib.simmd_profile_get(self.ctx, _lib.ptr(out)))
        return dict(force_ms=out[0], force_n=int(out[1]), kick_ms=out[2], rebuild_ms=out[3], update_ms=out[4],
                    steps=int(out[5]))

    def set_prune(self, inner_skin: float, rid: int = -1):
        """inner (pruned) lists for the force pass with this inner skin for
        one replica (rid) or all (-1); 0 everywhere turns them off"""
        _lib.check(self.lib.simmd_set_prune(self.ctx, rid, float(inner_skin)))
        if rid == -1:
            self.inner_skin = float(inner_skin)
        else:
            self.inner_skin = max(self.inner_skin, float(inner_skin))

    def prune_stats(self, rid: int):
        """(prunes done, inner-list entries at the last prune)"""
        n, e = C.c_int64(0), C.c_int64(0)
        _lib.check(self.lib.simmd_prune_stats(self.ctx, rid, C.byref(n), C.byref(e)))
        return n.value, e.value

    def set_skin(self, skin: float, rid: int = -1):
        _lib.check(self.lib.simmd_set_skin(self.ctx, rid, skin))
        for k, s in self.specs.items():
            if rid in (-1, k):
                s.skin = skin

    def set_tuning(self, tpp: int, graphs: bool = True, graph_steps: int = 16):
        _lib.check(self.lib.simmd_set_tuning(self.ctx, tpp, int(graphs), graph_steps))

    def set_work_item(self, particles: int):
        """force-pass tile shape: particles per work item (128, 64, 32; 0 = automatic)"""
        _lib.check(self.lib.simmd_set_work_item(self.ctx, int(particles)))

    def close(self):
        if self.ctx:
            self.lib.simmd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        self.close()
