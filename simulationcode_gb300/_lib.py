"""ctypes binding of libsimmd.so (the C ABI declared in include/simmd.h).

The library is built in-tree by ``simulationcode_gb300.build.build()``.  There
is no CPU fallback: if the shared library is missing this module raises, and
every compute call goes through the CUDA kernels of the library.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsimmd.so")

OK = 0
ERR_BAD_ARG, ERR_CUDA, ERR_OOM, ERR_NEIGHBOR_OVERFLOW, ERR_NONFINITE = 1, 2, 3, 4, 5
ERR_NOISE_RANGE, ERR_BUDGET, ERR_NOT_FOUND, ERR_NO_DEVICE, ERR_NOT_CONVERGED = 6, 7, 8, 9, 10

POT_LJ, POT_BERTHIER = 0, 1
NEWTONIAN, LANGEVIN, BROWNIAN = 0, 1, 2
FP64, FP32_SPLIT = 0, 1


class SimMDError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("libsimmd status %d: %s" % (status, message))
        self.status = status


class Params(C.Structure):
    """simmd_params (include/simmd.h)."""
    _fields_ = [
        ("dims", C.c_int32), ("potential", C.c_int32), ("dynamics", C.c_int32), ("precision", C.c_int32),
        ("N", C.c_int64),
        ("box_size", C.c_double), ("force_cutoff2", C.c_double), ("skin", C.c_double),
        ("verlet_force_cutoff", C.c_double),
        ("lj_eps", C.c_double), ("lj_sigma", C.c_double), ("lj_Uc", C.c_double),
        ("b_c0", C.c_double), ("b_c2", C.c_double), ("b_c4", C.c_double), ("b_zeta", C.c_double),
        ("kBT", C.c_double), ("gamma", C.c_double), ("dt", C.c_double), ("m", C.c_double),
        ("rescale_temperature", C.c_int32), ("max_neighbors", C.c_int32),
        ("seed", C.c_uint64),
    ]


class Stats(C.Structure):
    """simmd_stats (include/simmd.h)."""
    _fields_ = [
        ("steps_done", C.c_int64), ("rebuilds", C.c_int64), ("noise_draws", C.c_int64),
        ("max_neighbors", C.c_int32), ("max_count", C.c_int32), ("overflow", C.c_int32),
        ("nonfinite", C.c_int32),
        ("epot", C.c_double), ("virial", C.c_double), ("ekin", C.c_double),
        ("list_entries", C.c_int64),
    ]


# every symbol include/simmd.h declares, with (restype, argtypes)
_vp = C.c_void_p
_P = C.POINTER
SIGNATURES = {
    "simmd_version": (C.c_char_p, []),
    "simmd_status_string": (C.c_char_p, [C.c_int]),
    "simmd_last_error": (C.c_char_p, []),
    "simmd_device_count": (C.c_int, [_P(C.c_int32)]),
    "simmd_create": (C.c_int, [_P(Params), _P(_vp)]),
    "simmd_destroy": (C.c_int, [_vp]),
    "simmd_upload": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "simmd_download": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "simmd_set_state": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "simmd_set_state_r": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp, _vp]),
    "simmd_rebuild": (C.c_int, [_vp]),
    "simmd_forces": (C.c_int, [_vp, _vp, _vp]),
    "simmd_step": (C.c_int, [_vp, C.c_int64, _vp]),
    "simmd_energy": (C.c_int, [_vp, _P(C.c_double), _P(C.c_double), _P(C.c_double)]),
    "simmd_potential_energy_array": (C.c_int, [_vp, _vp]),
    "simmd_export_pairs": (C.c_int, [_vp, C.c_int32, C.c_int64, _vp, _vp]),
    "simmd_set_full_list": (C.c_int, [_vp, C.c_int32]),
    "simmd_stats_get": (C.c_int, [_vp, _P(Stats)]),
    "simmd_engine_create": (C.c_int, [C.c_int32, _P(_vp)]),
    "simmd_reserve": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int32, C.c_int32]),
    "simmd_add_replica": (C.c_int, [_vp, _P(Params), _vp, _vp, _vp, _vp, _P(C.c_int32)]),
    "simmd_remove_replica": (C.c_int, [_vp, C.c_int32]),
    "simmd_upload_r": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp, _vp, _vp]),
    "simmd_download_r": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp, _vp]),
    "simmd_transfer_layout": (C.c_int64, [_vp, C.c_int32, _vp]),
    "simmd_upload_all": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "simmd_download_all": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "simmd_set_state_all": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "simmd_energy_all": (C.c_int, [_vp]),
    "simmd_stats_r": (C.c_int, [_vp, C.c_int32, _P(Stats)]),
    "simmd_replica_bytes": (C.c_int64, [_P(Params), C.c_int32]),
    "simmd_set_tuning": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32]),
    "simmd_set_work_item": (C.c_int, [_vp, C.c_int32]),
    "simmd_set_skin": (C.c_int, [_vp, C.c_int32, C.c_double]),
    "simmd_set_prune": (C.c_int, [_vp, C.c_int32, C.c_double]),
    "simmd_prune_stats": (C.c_int, [_vp, C.c_int32, _vp, _vp]),
    "simmd_sync": (C.c_int, [_vp]),
    "simmd_stream": (_vp, [_vp]),
    "simmd_timer_start": (C.c_int, [_vp]),
    "simmd_timer_stop": (C.c_int, [_vp, _P(C.c_float)]),
    "simmd_launch_count": (C.c_int64, [_vp]),
    "simmd_kernel_counts": (C.c_int, [_vp, _P(C.c_int64), _P(C.c_int64)]),
    "simmd_device_bytes": (C.c_int64, [_vp]),
    "simmd_set_budget": (C.c_int, [_vp, C.c_int64]),
    "simmd_dump_async": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp]),
    "simmd_dump_wait": (C.c_int, [_vp]),
    "simmd_inherent_structure": (C.c_int, [_vp, C.c_double, C.c_int64, C.c_double, C.c_double, _P(C.c_int64)]),
    "simmd_time_force": (C.c_int, [_vp, C.c_int32, _P(C.c_float)]),
    "simmd_set_profile": (C.c_int, [_vp, C.c_int32]),
    "simmd_relax": (C.c_int, [_vp, C.c_int64, C.c_double, C.c_double]),
    "simmd_mc_sweeps": (C.c_int, [_vp, C.c_int64, C.c_double, C.c_double]),
    "simmd_mc_stats": (C.c_int, [_vp, C.c_int32, _vp, _P(C.c_double)]),
    "simmd_download_diameters": (C.c_int, [_vp, C.c_int32, _vp]),
    "simmd_host_register": (C.c_int, [_vp, C.c_int64]),
    "simmd_host_unregister": (C.c_int, [_vp]),
    "simmd_energy_virial_noalloc": (C.c_int, [_P(Params), _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp]),
    "simmd_profile_get": (C.c_int, [_vp, _vp]),
    "simmd_check_conversions": (C.c_int, [C.c_int64, C.c_uint64, _P(C.c_int64)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libsimmd.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libsimmd.so not found at %s: build it with "
                          "simulationcode_gb300.build.build() (no CPU fallback exists)" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != OK:
        lib = load()
        msg = lib.simmd_last_error().decode(errors="replace")
        raise SimMDError(status, msg or lib.simmd_status_string(status).decode())
    return status


def ptr(a):
    if a is None:
        return None
    if not (a.flags["C_CONTIGUOUS"]):
        raise ValueError("array must be C-contiguous")
    return C.c_void_p(a.ctypes.data)


def f64(a, shape=None):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def device_count() -> int:
    n = C.c_int32(0)
    load().simmd_device_count(C.byref(n))
    return n.value
