"""Minimal stand-in for the ``simulacra`` package, used ONLY to import the
reference ionization library in this container so that golden fixtures can be
generated from it (``tests/golden/make_golden.py``).

``simulacra`` is an unpinned runtime dependency of the reference
(requirements.txt lists the bare name) and is not available here.  This stub
supplies exactly the pieces the reference's mesh time-evolution path touches:
``Specification``/``Simulation`` (to_sim), ``Info``, ``Status``, the ``utils``
helpers (memoize, StrEnum, find_nearest_entry, ...), ``math.SphericalHarmonic``
and a permissive ``vis`` namespace.  Units are atomic units (``units.py``).
"""

import enum
import pickle
import uuid

from . import units, utils, math, vis  # noqa: F401


class Status(enum.Enum):
    INITIALIZED = "initialized"
    RUNNING = "running"
    PAUSED = "paused"
    FINISHED = "finished"
    ERROR = "error"


class Info:
    def __init__(self, *, header: str = ""):
        self.header = header
        self.children = []

    def add_field(self, name, value):
        self.children.append((name, value))

    def add_fields(self, fields):
        for name, value in fields:
            self.add_field(name, value)

    def add_info(self, info):
        self.children.append(info)

    def __str__(self):
        lines = [str(self.header)]
        for c in self.children:
            if isinstance(c, Info):
                lines.extend("  " + line for line in str(c).splitlines())
            else:
                lines.append(f"  {c[0]}: {c[1]}")
        return "\n".join(lines)


class Specification:
    simulation_type = None

    def __init__(self, name, file_name=None, **kwargs):
        self.name = str(name)
        self.file_name = file_name if file_name is not None else self.name
        self._extra_args = kwargs
        for k, v in kwargs.items():
            setattr(self, k, v)

    def to_sim(self):
        return self.simulation_type(self)

    def info(self):
        return Info(header=f"Specification: {self.name}")


class Simulation:
    def __init__(self, spec):
        self.spec = spec
        self.name = spec.name
        self.file_name = spec.file_name
        self.uuid = uuid.uuid4()
        self.status = Status.INITIALIZED

    def __hash__(self):
        return hash(self.uuid)

    def __eq__(self, other):
        return self is other

    def info(self):
        return Info(header=f"Simulation: {self.name}")

    def save(self, target_dir=None, **kwargs):
        import os

        target_dir = target_dir or os.getcwd()
        path = os.path.join(target_dir, f"{self.file_name}.sim")
        with open(path, "wb") as f:
            pickle.dump(self, f)
        return path

    @classmethod
    def load(cls, path):
        with open(path, "rb") as f:
            return pickle.load(f)
