"""Device probes of libsimmd (not on the simulation path).

``pipe_rates()`` measures, on the current GPU, the throughput of the FP64
adder, the float <-> double converters, the split-precision kernels' bit-level
conversions and the FP32 FMA pipe (G operations/s); ``check_conversions()``
runs the device self-check of those bit-level conversions and of the integer
grid index.  ``python -m simulationcode_gb300.devinfo`` prints both as one
JSON line.
"""
import ctypes as C
import json

import numpy as np

from . import _lib

RATE_NAMES = ("fp64_add", "f2d_converter", "f2d_bits", "d2f_converter", "d2f_bits", "fp32_fma")


def pipe_rates() -> dict:
    lib = _lib.load()
    out = np.zeros(6)
    _lib.check(lib.simmd_pipe_rates(_lib.ptr(out)))
    return {k: float(v) for k, v in zip(RATE_NAMES, out)}


def check_conversions(n: int = 1 << 24, seed: int = 1) -> int:
    lib = _lib.load()
    bad = C.c_int64(-1)
    _lib.check(lib.simmd_check_conversions(n, seed, C.byref(bad)))
    return bad.value


def main():
    rates = pipe_rates()
    print(json.dumps({"gops": {k: round(v, 1) for k, v in rates.items()},
                      "conversion_mismatches": check_conversions()}))


if __name__ == "__main__":
    main()
