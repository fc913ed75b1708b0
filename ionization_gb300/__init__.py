"""ionization_gb300 — GB300 (sm_103a) mesh time-evolution for ionization.

A drop-in for the mesh time-evolution path of the ionization library: the
same specification -> ``to_sim()`` -> ``run()`` API, mesh operator and
evolution-method classes, with every step executed by hand-written CUDA
kernels behind the C ABI of ``include/ionization_gb300.h``.
"""

from . import core, exceptions, potentials, states, units  # noqa: F401
from ._build import build  # noqa: F401
from .core import Gauge, Precision  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # submodules that import torch are loaded on first use
    if name in ("mesh", "cy", "batch", "serve"):
        import importlib

        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
