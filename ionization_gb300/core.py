"""Small shared types (ionization/core.py:121-129)."""

import dataclasses
import enum


class StrEnum(str, enum.Enum):
    def __str__(self):
        return str(self.value)


@dataclasses.dataclass(frozen=True)
class WarningRecord:
    data_time_index: int
    message: str


class Gauge(StrEnum):
    LENGTH = "LEN"
    VELOCITY = "VEL"


class Precision(StrEnum):
    """Arithmetic of the wavefunction and its sweeps on the device.

    C128: complex128 state and FP64 arithmetic (matches the reference).
    C64: complex64 state, FP32 sweeps, FP64 fields, coefficients and
    reductions.
    C64X: as C64, with the rounding residual of the state kept beside it
    (two bf16 a point, 12 bytes a point in all) and refined radial solves
    whose residual is formed with the FP64 Hamiltonian: storing the state no
    longer rounds it to FP32 and the FP32 coefficient tables no longer
    perturb the dynamics, which removes the dominant errors of C64."""

    C128 = "c128"
    C64 = "c64"
    C64X = "c64x"


@dataclasses.dataclass(frozen=True)
class SphericalHarmonic:
    """Y_l^m, the key of the per-l datastores (simulacra's SphericalHarmonic
    in the reference; only l and m matter here)."""

    l: int = 0
    m: int = 0

    def __str__(self):
        return f"Y_{self.l}^{self.m}"
