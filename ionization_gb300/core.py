"""Small shared types (ionization/core.py:121-129)."""

import dataclasses
import enum

import numpy as np


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


class LazyArray:
    """An array formed by ``make()`` when it is first read (``np.asarray``
    or any numpy call on it), then kept.  Host tables that only some forms
    upload (the complex128 radial diagonal over the whole (l, r) mesh, the
    full initial psi of which only the nonzero rows go up) are formed only
    where they are read."""

    __slots__ = ("_make", "_value")

    def __init__(self, make):
        self._make, self._value = make, None

    def value(self) -> np.ndarray:
        if self._value is None:
            self._value = np.asarray(self._make())
            self._make = None
        return self._value

    def __array__(self, dtype=None, copy=None):
        v = self.value()
        if dtype is not None and np.dtype(dtype) != v.dtype:
            return v.astype(dtype)
        return v.copy() if copy else v

    # indexing and the array's own attributes (shape, dtype, reshape, ...)
    def __getitem__(self, key):
        return self.value()[key]

    def __len__(self):
        return len(self.value())

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        return getattr(self.value(), name)
