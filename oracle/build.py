"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/simmd_oracle.c with gcc into oracle/_build/libsimmd_oracle.so.
-ffp-contract=off keeps every floating-point expression rounded as written
(no FMA contraction), which the bit-level parity of pair distances relies on.

The reference (SimulationCode.jl) is pure Julia and Julia is not installed,
so there is no oracle/_ref build of the reference itself.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsimmd_oracle.so")
SRC = os.path.join(HERE, "simmd_oracle.c")


def build_oracle(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "simmd_oracle.h")))):
        return LIB
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-D_DEFAULT_SOURCE", "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force=True))
