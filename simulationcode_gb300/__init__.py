"""simulationcode_gb300 -- SimulationCode.jl's molecular-dynamics hot path on
GB300 (sm_103a): neighbour-list rebuild and skin trigger, LJ and polydisperse
soft-sphere forces / energies / virial, Newtonian, Langevin and Brownian
updates, as hand-written CUDA kernels behind the C ABI of include/simmd.h.

This package is the host-side mirror of the reference's Julia interface
(same struct and function names) plus the multi-replica batch and serving
front ends.  Compute always runs in libsimmd.so; there is no CPU fallback.
"""
from .structs import (ArrayStruct, Berthier, Brownian, DumpInfo, LJ, Langevin, Newtonian, OutputStruct,
                      ParameterStruct, generate_diameters_)

__all__ = ["ArrayStruct", "Berthier", "Brownian", "DumpInfo", "LJ", "Langevin", "Newtonian", "OutputStruct",
           "ParameterStruct", "generate_diameters_"]


def __getattr__(name):
    # the device-backed API loads libsimmd.so on first use
    if name in ("md", "batch", "serving", "autotune"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)
