"""Quantum states used as initial and test states (host FP64).

Restates the parts of ionization/states/ the mesh path needs:
QuantumState (state.py:52-213), Superposition, HydrogenBoundState
(three_d.py:298-400).  ``GaussianState`` has no reference class; it is the
user QuantumState subclass the 1D Gaussian workload needs.
"""

import abc
import functools
from copy import deepcopy

import numpy as np
import scipy.special as special

from .. import core, exceptions, summables
from .. import units as u


class Eigenvalues(core.StrEnum):
    DISCRETE = "discrete"
    CONTINUOUS = "continuous"


class Binding(core.StrEnum):
    BOUND = "bound"
    FREE = "free"


class Derivation(core.StrEnum):
    ANALYTIC = "analytic"
    NUMERIC = "numeric"
    VARIATIONAL = "variational"


class QuantumState(summables.Summand, abc.ABC):
    eigenvalues = None
    binding = None
    derivation = None

    def __init__(self, amplitude=1):
        super().__init__()
        self.amplitude = amplitude
        self.summation_class = Superposition

    @property
    def numeric(self):
        return self.derivation == Derivation.NUMERIC

    @property
    def analytic(self):
        return self.derivation == Derivation.ANALYTIC

    @property
    def bound(self):
        return self.binding == Binding.BOUND

    @property
    def free(self):
        return self.binding == Binding.FREE

    @property
    def norm(self):
        return np.abs(self.amplitude) ** 2

    def __mul__(self, other):
        new = deepcopy(self)
        new.amplitude *= other
        return new

    def __rmul__(self, other):
        return self * other

    def __truediv__(self, other):
        return self * (1 / other)

    @property
    @abc.abstractmethod
    def tuple(self):
        raise NotImplementedError

    def __hash__(self):
        return hash((self.__class__.__name__,) + self.tuple)

    def __eq__(self, other):
        return isinstance(other, self.__class__) and self.tuple == other.tuple

    def __lt__(self, other):
        return isinstance(other, self.__class__) and self.tuple < other.tuple

    def __gt__(self, other):
        return isinstance(other, self.__class__) and self.tuple > other.tuple

    @abc.abstractmethod
    def __call__(self, *args, **kwargs):
        raise NotImplementedError

    def __str__(self):
        return self.ket

    @property
    def ket(self):
        return f"|{self.__class__.__name__}>"


class Superposition(summables.Sum, QuantumState):
    container_name = "states"

    def __init__(self, *states):
        norm = np.sqrt(sum(s.norm for s in states))
        super().__init__(*(s / norm for s in states), amplitude=1)

    @property
    def tuple(self):
        return tuple(sorted(s.tuple for s in self.states))

    def __call__(self, *args, **kwargs):
        return sum(s(*args, **kwargs) for s in self.states)


class SphericalHarmonicState(QuantumState):
    def __init__(self, l=0, m=0, amplitude=1):
        super().__init__(amplitude=amplitude)
        self.l = l
        self.m = m

    @property
    def spherical_harmonic(self):
        return (self.l, self.m)

    @abc.abstractmethod
    def radial_function(self, r):
        raise NotImplementedError

    def __call__(self, r, theta, phi):
        """amplitude * R(r) * Y_l^m(theta, phi)  (three_d.py:198-203)."""
        return self.amplitude * self.radial_function(r) * special.sph_harm_y(self.l, self.m, theta, phi)


class HydrogenBoundState(SphericalHarmonicState):
    eigenvalues = Eigenvalues.DISCRETE
    binding = Binding.BOUND
    derivation = Derivation.ANALYTIC

    def __init__(self, n=1, l=0, m=0, amplitude=1):
        bad = None
        if int(n) != n or n < 1:
            bad = f"principal quantum number n = {n} is not a positive integer"
        elif int(l) != l or not 0 <= l < n:
            bad = f"angular momentum l = {l} is not an integer in [0, {n}) for n = {n}"
        elif int(m) != m or abs(m) > l:
            bad = f"magnetic quantum number m = {m} is not an integer in [-{l}, {l}]"
        if bad:
            raise exceptions.IllegalQuantumState(bad)
        self.n = int(n)
        super().__init__(l=int(l), m=int(m), amplitude=amplitude)

    @property
    def energy(self):
        return -u.rydberg / (self.n ** 2)

    @property
    def tuple(self):
        return self.n, self.l, self.m

    def __repr__(self):
        return f"HydrogenBoundState(n = {self.n}, l = {self.l}, m = {self.m}, amplitude = {self.amplitude})"

    @property
    def ket(self):
        return f"|{self.n},{self.l},{self.m}>"

    def radial_function(self, r):
        """Griffiths-normalised radial function (three_d.py:375-391)."""
        n, l = self.n, self.l
        normalization = _bound_normalization(n, l)
        r_dep = np.exp(-r / (n * u.bohr_radius)) * ((2 * r / (n * u.bohr_radius)) ** l)
        lag_poly = special.eval_genlaguerre(n - l - 1, (2 * l) + 1, 2 * r / (n * u.bohr_radius))
        return self.amplitude * normalization * r_dep * lag_poly


@functools.lru_cache(maxsize=None)
def _bound_normalization(n, l):
    """The radial function's normalisation constant, formed once per (n, l)
    (the same expression every call; scipy's factorial is slow to call)."""
    return np.sqrt(
        ((2 / (n * u.bohr_radius)) ** 3)
        * (special.factorial(n - l - 1) / (2 * n * special.factorial(n + l)))
    )


def electron_wavenumber_from_energy(energy):
    """core.py:19-20."""
    return np.sqrt(2 * u.electron_mass * np.abs(energy)) / u.hbar


class HydrogenCoulombState(SphericalHarmonicState):
    """A hydrogen free state labelled by its energy (states/three_d.py:414-470);
    here it names the free numeric eigenstates."""

    eigenvalues = Eigenvalues.CONTINUOUS
    binding = Binding.FREE
    derivation = Derivation.ANALYTIC

    def __init__(self, energy=1 * u.eV, l=0, m=0, amplitude=1.0):
        if energy < 0:
            raise exceptions.IllegalQuantumState(f"a free state's energy cannot be negative (got {energy})")
        self.energy = energy
        super().__init__(l=l, m=m, amplitude=amplitude)

    @property
    def wavenumber(self):
        return electron_wavenumber_from_energy(self.energy)

    @property
    def tuple(self):
        return self.wavenumber, self.l, self.m, self.energy

    def radial_function(self, r):
        raise NotImplementedError("Coulomb radial functions are not evaluated here; use the numeric eigenbasis")

    def __repr__(self):
        return f"HydrogenCoulombState(energy = {self.energy}, l = {self.l}, m = {self.m})"


class NumericSphericalHarmonicState(SphericalHarmonicState):
    """A numerically derived radial state (states/three_d.py:543-630): its
    radial function is the stored vector ``g``, labelled by the analytic
    state it approximates."""

    eigenvalues = Eigenvalues.DISCRETE
    derivation = Derivation.NUMERIC

    def __init__(self, *, g, l=0, m=0, energy, corresponding_analytic_state, binding, amplitude=1):
        self.g = g
        self.energy = energy
        self.corresponding_analytic_state = corresponding_analytic_state
        self.binding = binding
        super().__init__(l=l, m=m, amplitude=amplitude)

    @property
    def n(self):
        return self.corresponding_analytic_state.n

    @property
    def wavenumber(self):
        return self.corresponding_analytic_state.wavenumber

    @property
    def tuple(self):
        return self.corresponding_analytic_state.tuple

    def radial_function(self, r):
        return self.g

    def __repr__(self):
        return repr(self.corresponding_analytic_state) + "_n"

    @property
    def ket(self):
        return self.corresponding_analytic_state.ket + "_n"


class GaussianState(QuantumState):
    """exp(-(z - center)^2 / (2 width^2)), normalised on the mesh when
    projected (a 1D bound wavepacket; user-state extension)."""

    eigenvalues = Eigenvalues.DISCRETE
    binding = Binding.BOUND
    derivation = Derivation.ANALYTIC

    def __init__(self, width=1.0, center=0.0, amplitude=1):
        self.width = width
        self.center = center
        super().__init__(amplitude=amplitude)

    @property
    def tuple(self):
        return (self.width, self.center)

    def __call__(self, z):
        return np.exp(-((z - self.center) ** 2) / (2 * self.width ** 2)).astype(np.complex128)

    def __repr__(self):
        return f"GaussianState(width = {self.width}, center = {self.center})"


class TwoDGaussianWavepacket(QuantumState):
    """A free 2D Gaussian wavepacket in (z, x) (states/two_d.py:259-315):
    exp(-(z - z0)^2 / (2 wz^2)) exp(-(x - x0)^2 / (2 wx^2)) exp(i (kz z + kx x))
    / (sqrt(2 pi) sqrt(wz wx)), evaluated at (r, theta) as z = r cos theta,
    x = r sin theta."""

    eigenvalues = Eigenvalues.CONTINUOUS
    binding = Binding.FREE
    derivation = Derivation.ANALYTIC

    def __init__(self, center_z=0, center_x=0, width_z=1 * u.nm, width_x=1 * u.nm, k_z=0, k_x=0,
                 mass=u.electron_mass, amplitude=1):
        if width_z <= 0:
            raise exceptions.InvalidQuantumStateParameter("width_z must be positive")
        if width_x <= 0:
            raise exceptions.InvalidQuantumStateParameter("width_x must be positive")
        self.center_z, self.center_x = center_z, center_x
        self.width_z, self.width_x = width_z, width_x
        self.k_z, self.k_x = k_z, k_x
        self.mass = mass
        super().__init__(amplitude=amplitude)

    @property
    def tuple(self):
        return self.center_z, self.center_x, self.width_z, self.width_x

    def eval_z_x(self, z, x):
        norm = 1 / (np.sqrt(u.twopi) * np.sqrt(self.width_z * self.width_x))
        gaussian = np.exp(-0.5 * (((z - self.center_z) / self.width_z) ** 2)) * np.exp(
            -0.5 * (((x - self.center_x) / self.width_x) ** 2))
        return norm * gaussian * (np.exp(1j * self.k_z * z) * np.exp(1j * self.k_x * x))

    def eval_r_theta(self, r, theta):
        return self.eval_z_x(r * np.cos(theta), r * np.sin(theta))

    def __call__(self, r, theta):
        return self.eval_r_theta(r, theta)

    def __repr__(self):
        return (f"TwoDGaussianWavepacket(center_z = {self.center_z}, center_x = {self.center_x}, width_z = "
                f"{self.width_z}, width_x = {self.width_x}, k_z = {self.k_z}, k_x = {self.k_x})")
