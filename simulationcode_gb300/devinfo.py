"""Device self-check of libsimmd (not on the simulation path).

``check_conversions()`` runs, on the current GPU, the self-check of the
split-precision kernels' bit-level float <-> double conversions against the
hardware converter (0 mismatches expected).  ``python -m simulationcode_gb300.devinfo`` prints
the count as one JSON line.
"""
import ctypes as C
import json

from . import _lib


def check_conversions(n: int = 1 << 24, seed: int = 1) -> int:
    lib = _lib.load()
    bad = C.c_int64(-1)
    _lib.check(lib.simmd_check_conversions(n, seed, C.byref(bad)))
    return bad.value


def main():
    print(json.dumps({"conversion_mismatches": check_conversions()}))


if __name__ == "__main__":
    main()
