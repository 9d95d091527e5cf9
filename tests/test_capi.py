"""The C-ABI library builds, loads and exports every symbol of include/simmd.h
(CPU-only checks: no kernel is launched)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "simmd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(simmd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_abi():
    syms = declared_symbols()
    for s in ("simmd_create", "simmd_rebuild", "simmd_forces", "simmd_step", "simmd_energy",
              "simmd_export_pairs", "simmd_add_replica"):
        assert s in syms


def test_library_exports_every_declared_symbol(simlib):
    missing = [s for s in declared_symbols() if not hasattr(simlib, s)]
    assert not missing, missing


def test_python_binding_covers_every_symbol(simlib):
    from simulationcode_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_params_struct_layout_matches_header():
    from simulationcode_gb300 import _lib
    # 4 int32 + int64 + 15 doubles + 2 int32 + uint64
    assert C.sizeof(_lib.Params) == 4 * 4 + 8 + 15 * 8 + 2 * 4 + 8
    assert C.sizeof(_lib.Stats) == 3 * 8 + 4 * 4 + 3 * 8 + 8


def test_status_strings_and_no_device_error(simlib):
    from simulationcode_gb300 import _lib
    assert simlib.simmd_status_string(4) == b"neighbour list overflow"
    assert simlib.simmd_version().startswith(b"simmd")
    n = C.c_int32(-1)
    assert simlib.simmd_device_count(C.byref(n)) == 0
    if n.value == 0:
        ctx = C.c_void_p()
        assert simlib.simmd_engine_create(0, C.byref(ctx)) == _lib.ERR_NO_DEVICE
        assert not ctx.value


def test_bad_parameters_rejected_before_any_device_work(simlib):
    from simulationcode_gb300 import _lib
    p = _lib.Params()
    p.dims = 4
    p.N = 10
    ctx = C.c_void_p()
    assert simlib.simmd_create(C.byref(p), C.byref(ctx)) == _lib.ERR_BAD_ARG
    assert b"dims" in simlib.simmd_last_error()


def test_replica_bytes_estimate(simlib):
    from simulationcode_gb300 import _lib
    p = _lib.Params()
    p.N = 4096
    b = simlib.simmd_replica_bytes(C.byref(p), 64)
    assert 4096 * 256 < b < 4096 * 2048


def test_noalloc_entry_rejects_before_any_device_work(simlib):
    """the no-allocation entry point checks its sizes before it touches a
    device: N beyond its fixed scratch is SIMMD_ERR_BUDGET, with the limit
    named in simmd_last_error"""
    from simulationcode_gb300 import _lib
    buf = (C.c_double * 8)()
    ptrs = [C.cast(buf, C.c_void_p)] * 5
    p = _lib.Params()
    p.dims, p.potential = 3, 1
    p.N = 1048576 + 1
    st = simlib.simmd_energy_virial_noalloc(C.byref(p), *ptrs[:4], 1, ptrs[4], None)
    assert st == _lib.ERR_BUDGET
    assert b"SIMMD_NOALLOC_MAX_N" in simlib.simmd_last_error()
    p.N = 0
    assert simlib.simmd_energy_virial_noalloc(C.byref(p), *ptrs[:4], 1, ptrs[4], None) == _lib.ERR_BAD_ARG
    p.N, p.dims = 10, 4
    assert simlib.simmd_energy_virial_noalloc(C.byref(p), *ptrs[:4], 1, ptrs[4], None) == _lib.ERR_BAD_ARG
    assert b"dims" in simlib.simmd_last_error()
