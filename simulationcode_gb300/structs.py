"""Host-side mirror of SimulationCode.jl's data model (src/DataStructs.jl).

Same names, fields and meaning as the Julia structs, so code written against
the reference reads the same here.  Arrays are numpy in the reference's
ArrayStruct layout: ``(N, dims)`` float64 rows = Julia's SVector columns.
"""
from __future__ import annotations

import dataclasses
from typing import Any, Callable, Optional, Sequence

import numpy as np


@dataclasses.dataclass
class LJ:
    """LJ(eps, sigma, rc) with shift Uc = 4eps((sigma/rc)^12 - (sigma/rc)^6)
    (src/DataStructs.jl:10-19)."""
    eps: float
    sigma: float
    rc: float
    Uc: float = dataclasses.field(init=False)

    def __post_init__(self):
        x = self.sigma / self.rc
        self.Uc = 4 * self.eps * (x ** 12 - x ** 6)


@dataclasses.dataclass
class Berthier:
    """Polydisperse soft spheres, Berthier(; n=12, rc=1.25, sigma_ratio=2.219,
    zeta=0.2) (src/DataStructs.jl:45-60)."""
    n: int = 12
    rc: float = 1.25
    sigma_ratio: float = 2.219
    zeta: float = 0.2
    c0: float = dataclasses.field(init=False)
    c2: float = dataclasses.field(init=False)
    c4: float = dataclasses.field(init=False)

    def __post_init__(self):
        if self.n != 12:
            raise AssertionError("Berthier potential requires n == 12")
        n, rc = self.n, self.rc
        self.c0 = -(1 / 8) * (8 + 6 * n + n ** 2) * rc ** -n
        self.c2 = 1 / 4 * n * (4 + n) * rc ** (-2 - n)
        self.c4 = -(1 / 8) * n * (2 + n) * rc ** (-4 - n)


@dataclasses.dataclass
class Newtonian:
    """Newtonian(kBT, dt, m, rescale_temperature, dims) (src/DataStructs.jl:71-77)."""
    kBT: float
    dt: float
    m: float
    rescale_temperature: bool
    dims: int


@dataclasses.dataclass
class Langevin:
    """Langevin(kBT, gamma, dt, m, dims); rescale_temperature always False
    (src/DataStructs.jl:79-87)."""
    kBT: float
    gamma: float
    dt: float
    m: float
    dims: int
    rescale_temperature: bool = False


@dataclasses.dataclass
class Brownian:
    """Brownian(kBT, gamma, dt, dims) (src/DataStructs.jl:64-69)."""
    kBT: float
    gamma: float
    dt: float
    dims: int


@dataclasses.dataclass
class DumpInfo:
    """DumpInfo (src/DataStructs.jl:90-99).  ``writer`` (an addition) receives
    (step, dict of arrays) at every dump step; the reference writes HDF5."""
    save: bool
    filename: str
    when_to_save_array: Sequence[int]
    save_r: bool = True
    save_v: bool = True
    save_F: bool = True
    save_D: bool = False
    save_Epot: bool = False
    writer: Optional[Callable[[int, dict], None]] = None

    def _when_set(self) -> frozenset:
        """when_to_save_array as a set (membership test of save_data)"""
        key = tuple(self.when_to_save_array)
        if getattr(self, "_when_key", None) != key:
            self._when_key = key
            self._when = frozenset(key)
        return self._when


@dataclasses.dataclass
class ParameterStruct:
    """ParameterStruct (src/DataStructs.jl:138-153)."""
    N_MD_equilibration_steps: int
    random_seed: int
    rho: float
    N: int
    box_size: float
    N_steps: int
    swap_probability: float
    max_MC_displacement: float
    force_cutoff2: float
    q_cutoff: float
    system: Any
    interaction_potential: Any
    dump_info: Optional[DumpInfo] = None
    callback: Optional[Callable] = None


class ArrayStruct:
    """ArrayStruct{dims} (src/DataStructs.jl:183-201): (N, dims) float64 arrays."""

    def __init__(self, N: int, dims: int):
        self.dims = dims
        self.r_array = np.zeros((N, dims))
        self.r_old_array = np.zeros((N, dims))
        self.D_array = np.zeros(N)
        self.v_array = np.zeros((N, dims))
        self.F_array = np.zeros((N, dims))
        self.random_displacement = np.zeros((N, dims))
        self.potential_energy_array = np.zeros(N)


@dataclasses.dataclass
class OutputStruct:
    """OutputStruct (src/DataStructs.jl:291-315)."""
    potential_energy: float = 0.0
    kinetic_energy: float = 0.0
    steps_done: int = 0
    N_translations_accepted: int = 0
    N_swaps_accepted: int = 0
    N_translations_total: int = 0
    N_swaps_total: int = 0
    N_neighbor_list_rebuilds: int = 0
    q4: float = 0.0
    q6: float = 0.0
    F2s: float = 0.0
    virial: float = 0.0


def generate_diameters_(arrays: ArrayStruct, parameters: ParameterStruct, U, rng=None):
    """generate_diameters! (src/InitialConfiguration.jl:1-18): Berthier
    diameters are regular inverse-CDF quantiles of P(D) ~ D^-3, shuffled;
    LJ diameters all sigma."""
    N = arrays.D_array.shape[0]
    if isinstance(U, Berthier):
        A = 1 / 2 + 1 / (U.sigma_ratio - 1)
        smin = (1 + U.sigma_ratio) / (2 * U.sigma_ratio)
        P = np.linspace(1 / (2 * N), 1 - 1 / (2 * N), N)
        D = np.sqrt(1 / (smin ** -2 - 2 * P / A))
        rng = rng if rng is not None else np.random.default_rng(parameters.random_seed)
        arrays.D_array[:] = rng.permutation(D)
    else:
        arrays.D_array[:] = U.sigma
