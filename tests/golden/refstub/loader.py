"""Import the reference ``ionization`` package read-only, for fixture generation.

Used only by ``tests/golden/make_golden.py`` in a container that has the
reference checkout.  It never runs on the GPU machine and nothing in the product
imports it.

What it does before ``import ionization``:
  * puts the ``simulacra`` stub (atomic units) first on ``sys.path``;
  * registers empty stand-ins for matplotlib / mpl_toolkits / cycler / htmap
    (plotting and HTCondor are not on the time-evolution path);
  * restores removed NumPy/SciPy aliases the reference still calls
    (``np.NaN``, ``scipy.integrate.simps``/``cumtrapz``, ``special.sph_harm``);
  * disables bytecode writing and redirects pyximport's build directory out of
    the reference tree, so the checkout is never written to.
"""

import os
import sys
import tempfile
import types

_HERE = os.path.dirname(os.path.abspath(__file__))


class _Anything(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _AnyObj()


class _AnyObj:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _AnyObj()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _AnyObj()


def _stub_module(name):
    mod = _Anything(name)
    mod.__file__ = None
    mod.__path__ = []
    sys.modules[name] = mod
    return mod


def import_reference(ref_root: str):
    sys.dont_write_bytecode = True
    os.environ["PYTHONDONTWRITEBYTECODE"] = "1"

    if _HERE not in sys.path:
        sys.path.insert(0, _HERE)

    for name in (
        "matplotlib",
        "matplotlib.pyplot",
        "matplotlib.colors",
        "matplotlib.cm",
        "matplotlib.patches",
        "matplotlib.animation",
        "mpl_toolkits",
        "mpl_toolkits.axes_grid1",
        "mpl_toolkits.mplot3d",
        "cycler",
        "htmap",
    ):
        if name not in sys.modules:
            _stub_module(name)

    import numpy as np
    import scipy.integrate as integ
    import scipy.special as special

    if not hasattr(np, "NaN"):
        np.NaN = np.nan
    if not hasattr(np, "Inf"):
        np.Inf = np.inf
    if not hasattr(integ, "simps"):
        integ.simps = integ.simpson
    if not hasattr(integ, "cumtrapz"):
        integ.cumtrapz = integ.cumulative_trapezoid
    if not hasattr(special, "sph_harm"):
        special.sph_harm = lambda m, l, phi, theta: special.sph_harm_y(l, m, theta, phi)

    import pyximport

    build_dir = os.path.join(tempfile.gettempdir(), "ion_ref_pyxbld")
    _orig_install = pyximport.install

    def _install(*args, **kwargs):
        kwargs["build_dir"] = build_dir
        return _orig_install(*args, **kwargs)

    pyximport.install = _install

    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)

    import ionization

    return ionization
