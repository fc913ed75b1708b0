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
    """Arithmetic of the wavefunction and its sweeps on the device."""

    C128 = "c128"
    C64 = "c64"
