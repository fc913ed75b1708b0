"""Potentials, pulses and masks evaluated on the host in FP64.

Restates the pieces of ionization/potentials/ that the mesh time-evolution
path consumes: the static internal potential V(r) (built once into the
Hamiltonian tables), the field amplitude E(t) (tabulated per time index and
uploaded once per run) and the mask m(r) (tabulated once).  Formulas and
operation order follow the reference so that tables are bit-identical.
"""

import operator

import numpy as np
import scipy.integrate as integ

from .. import exceptions, summables
from .. import units as u

# --------------------------------------------------------------------------
# potential energies (potentials/potential.py:14-70, static.py:12-110)
# --------------------------------------------------------------------------


class PotentialEnergy(summables.Summand):
    def __init__(self, *args, **kwargs):
        super().__init__()
        self.summation_class = PotentialEnergySum


class PotentialEnergySum(summables.Sum, PotentialEnergy):
    container_name = "potentials"

    def get_electric_field_amplitude(self, t):
        return sum(x.get_electric_field_amplitude(t) for x in self.members())

    def get_vector_potential_amplitude_numeric(self, times, rule="simps"):
        return sum(x.get_vector_potential_amplitude_numeric(times, rule=rule) for x in self.members())


class NoPotentialEnergy(PotentialEnergy):
    def __call__(self, r=None, *args, **kwargs):
        return np.zeros_like(r)


class CoulombPotential(PotentialEnergy):
    """k q Q / r  (potentials/static.py:12-51)."""

    def __init__(self, charge: float = 1 * u.proton_charge):
        super().__init__()
        self.charge = charge

    def __call__(self, *, r, test_charge, **kwargs):
        return u.coulomb_constant * self.charge * test_charge / r

    def __repr__(self):
        return f"CoulombPotential(charge = {self.charge})"


class SoftCoulombPotential(PotentialEnergy):
    """k q Q / sqrt(r^2 + s^2)  (potentials/static.py:54-110)."""

    def __init__(self, charge: float = 1 * u.proton_charge, softening_distance: float = 0.05 * u.bohr_radius):
        super().__init__()
        self.charge = charge
        self.softening_distance = softening_distance

    def __call__(self, *, r, test_charge, **kwargs):
        return (
            u.coulomb_constant
            * self.charge
            * test_charge
            / np.sqrt((r ** 2) + (self.softening_distance ** 2))
        )

    def __repr__(self):
        return f"SoftCoulombPotential(charge = {self.charge}, softening_distance = {self.softening_distance})"


# --------------------------------------------------------------------------
# time windows (potentials/windows.py:11-35)
# --------------------------------------------------------------------------


class TimeWindow(summables.Summand):
    def __init__(self):
        super().__init__()
        self.summation_class = TimeWindowSum


class TimeWindowSum(summables.Sum, TimeWindow):
    container_name = "windows"
    fold = staticmethod(operator.mul)  # windows multiply


class NoTimeWindow(TimeWindow):
    def __call__(self, t):
        return 1


# --------------------------------------------------------------------------
# electric potentials (potentials/pulses.py:19-97, 1696-1814)
# --------------------------------------------------------------------------


class ElectricPotential(PotentialEnergy):
    pass


class UniformLinearlyPolarizedElectricPotential(ElectricPotential):
    def __init__(self, window: TimeWindow = NoTimeWindow()):
        super().__init__()
        self.window = window

    def get_electric_field_amplitude(self, t):
        return self.window(t)

    def __call__(self, *, t, z, test_charge, **kwargs):
        """-z q E(t)  (pulses.py:37-56)."""
        return -z * test_charge * self.get_electric_field_amplitude(t)

    def get_electric_field_integral_numeric(self, times, rule: str = "simps"):
        y = self.get_electric_field_amplitude(times)
        if rule == "simps":
            return integ.simpson(y=y, x=times)
        return getattr(integ, rule)(y=y, x=times)

    def get_vector_potential_amplitude_numeric(self, times, rule: str = "simps"):
        """A at times[-1]: minus the integral of E (pulses.py:75-77)."""
        return -self.get_electric_field_integral_numeric(times, rule=rule)

    def get_electric_field_integral_numeric_cumulative(self, times):
        return integ.cumulative_trapezoid(y=self.get_electric_field_amplitude(times), x=times, initial=0)

    def get_vector_potential_amplitude_numeric_cumulative(self, times):
        return -self.get_electric_field_integral_numeric_cumulative(times)

    def __add__(self, other):
        return PotentialEnergySum(*self, *other)


class NoElectricPotential(UniformLinearlyPolarizedElectricPotential):
    def get_electric_field_amplitude(self, t):
        return np.zeros(np.shape(t)) * self.window(t)


DEFAULT_PHASE = 0
DEFAULT_PULSE_CENTER = 0


def _carrier_wavelength(omega):
    """Wavelength of angular frequency ``omega``: c / (omega / 2 pi)."""
    return u.c / (omega / u.twopi)


class CosSquaredPulse(UniformLinearlyPolarizedElectricPotential):
    """cos^2-envelope pulse parameterised by number of cycles
    (pulses.py:1696-1814).  Like the reference it stores the carrier as a
    wavelength and derives omega from it, so tabulated fields are identical."""

    def __init__(
        self,
        amplitude=0.01 * u.atomic_electric_field,
        wavelength=800 * u.nm,
        number_of_cycles=4,
        phase=DEFAULT_PHASE,
        pulse_center=DEFAULT_PULSE_CENTER,
        **kwargs,
    ):
        super().__init__(**kwargs)
        self.amplitude = amplitude
        self.wavelength_carrier = wavelength
        self.number_of_cycles = number_of_cycles
        self.phase = phase
        self.pulse_center = pulse_center

    @classmethod
    def from_omega_carrier(cls, amplitude=0.1 * u.atomic_electric_field, omega_carrier=u.twopi * u.c / (800 * u.nm),
                           number_of_cycles=4, phase=DEFAULT_PHASE, pulse_center=DEFAULT_PULSE_CENTER, **kwargs):
        """The pulse with angular carrier frequency ``omega_carrier``.  The
        carrier is kept as the wavelength c / (omega / 2 pi), and omega is
        recomputed from it, so E(t) matches the reference's to the last bit."""
        return cls(amplitude, _carrier_wavelength(omega_carrier), number_of_cycles, phase, pulse_center, **kwargs)

    @classmethod
    def from_sin2_envelope(cls, amplitude, omega, number_of_cycles, cep=0.0, t_start=0.0):
        """E0 sin^2(pi (t - t_start)/T) cos(omega (t - t_start) + cep), T = N 2 pi / omega.

        The carrier of CosSquaredPulse is centred on ``pulse_center``; with the
        centre at t_start + T/2 the phase is cep + N pi (mod 2 pi)."""
        T = number_of_cycles * u.twopi / omega
        return cls.from_omega_carrier(
            amplitude=amplitude,
            omega_carrier=omega,
            number_of_cycles=number_of_cycles,
            phase=float(np.mod(cep + np.pi * number_of_cycles, 2 * np.pi)),
            pulse_center=t_start + T / 2,
        )

    @property
    def frequency_carrier(self):
        return u.c / self.wavelength_carrier

    @property
    def period_carrier(self):
        return 1 / self.frequency_carrier

    @property
    def omega_carrier(self):
        return u.twopi * u.c / self.wavelength_carrier

    @property
    def pulse_width(self):
        return self.number_of_cycles * self.period_carrier

    @property
    def total_time(self):
        return self.period_carrier * self.number_of_cycles

    def get_electric_field_envelope(self, t):
        tau = t - self.pulse_center
        return np.where(
            np.less_equal(-self.total_time / 2, tau) * np.less_equal(tau, self.total_time / 2),
            np.cos(self.omega_carrier * tau / (2 * self.number_of_cycles)) ** 2,
            0,
        )

    def get_electric_field_amplitude(self, t):
        tau = t - self.pulse_center
        amp = self.get_electric_field_envelope(t) * np.cos((self.omega_carrier * tau) + self.phase)
        return amp * self.amplitude * super().get_electric_field_amplitude(t)

    def __repr__(self):
        return (
            f"CosSquaredPulse(amplitude = {self.amplitude}, omega = {self.omega_carrier}, "
            f"number_of_cycles = {self.number_of_cycles}, phase = {self.phase}, "
            f"pulse_center = {self.pulse_center})"
        )


def field_table(electric_potential, times):
    """E evaluated at every entry of ``times`` (FP64, host)."""
    return np.asarray(electric_potential.get_electric_field_amplitude(np.asarray(times)), dtype=np.float64) * np.ones(
        len(times)
    )


def simpson_prefix_integrals(y, x):
    """I[k] = the integral of y over x[:k+1] for every k, each by Simpson's rule
    for irregularly spaced samples as ``get_vector_potential_amplitude_numeric``
    evaluates it at every step (pulses.py:58-77 with ``integrate.simps``):
    k = 1, the trapezoid; an odd number of samples, the composite rule over
    pairs of intervals (h0, h1):
        (h0 + h1)/6 [y0 (2 - h1/h0) + y1 (h0 + h1)^2/(h0 h1) + y2 (2 - h0/h1)];
    an even number, the composite rule up to the last interval plus the
    parabola through the last three samples integrated over the last interval
    (Cartwright 2017):
        (2 h1^2 + 3 h0 h1)/(6 (h0 + h1)) y2 + (h1^2 + 3 h0 h1)/(6 h0) y1
        - h1^3/(6 h0 (h0 + h1)) y0.
    All prefixes in O(n) (a running sum of the pair terms) instead of one
    O(n) integral per step."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    out = np.zeros(n)
    if n < 2:
        return out
    h = np.diff(x)
    out[1] = 0.5 * h[0] * (y[0] + y[1])
    m = (n - 1) // 2  # whole pairs of intervals
    if m == 0:
        return out
    h0, h1 = h[0 : 2 * m : 2], h[1 : 2 * m : 2]
    hs, hp, q = h0 + h1, h0 * h1, h0 / h1
    pair = hs / 6.0 * (y[0 : 2 * m : 2] * (2.0 - 1.0 / q) + y[1 : 2 * m : 2] * (hs * hs / hp) + y[2 : 2 * m + 1 : 2] * (2.0 - q))
    cum = np.concatenate([[0.0], np.cumsum(pair)])
    k = np.arange(2, n, 2)  # odd sample counts
    out[k] = cum[k // 2]
    k = np.arange(3, n, 2)  # even sample counts
    a0, a1 = h[k - 2], h[k - 1]
    alpha = (2 * a1 ** 2 + 3 * a0 * a1) / (6 * (a1 + a0))
    beta = (a1 ** 2 + 3 * a0 * a1) / (6 * a0)
    eta = a1 ** 3 / (6 * a0 * (a0 + a1))
    out[k] = cum[(k - 1) // 2] + alpha * y[k] + beta * y[k - 1] - eta * y[k - 2]
    return out


def vector_potential_table(electric_potential, times):
    """A(times[k]) for every k: minus the integral of E over times[:k+1], the
    value the velocity-gauge operators take at step k (mesh_operators.py:
    1186-1196, 371-380, with sims.py:195-196)."""
    return -simpson_prefix_integrals(field_table(electric_potential, times), times)


# --------------------------------------------------------------------------
# masks (potentials/masks.py:11-113)
# --------------------------------------------------------------------------


class Mask(summables.Summand):
    def __init__(self):
        super().__init__()
        self.summation_class = MaskSum


class MaskSum(summables.Sum, Mask):
    container_name = "masks"
    fold = staticmethod(operator.mul)  # masks multiply


class NoMask(Mask):
    def __call__(self, *args, **kwargs):
        return 1


class RadialCosineMask(Mask):
    """|cos(pi/2 (r - r_in)/(r_out - r_in))|^(1/s) on [r_in, r_out), 0 beyond
    (masks.py:38-89).  On a line mesh ``r`` is the signed z, so this mask only
    absorbs at +z, as in the reference."""

    def __init__(self, inner_radius=50 * u.bohr_radius, outer_radius=100 * u.bohr_radius, smoothness=8):
        if min(inner_radius, outer_radius) < 0:
            raise exceptions.InvalidMaskParameter(
                f"mask radii cannot be negative (inner {inner_radius}, outer {outer_radius})")
        if not inner_radius < outer_radius:
            raise exceptions.InvalidMaskParameter(
                f"the mask's inner radius {inner_radius} is not below its outer radius {outer_radius}")
        if smoothness < 1:
            raise exceptions.InvalidMaskParameter(f"mask smoothness {smoothness} is below 1")
        super().__init__()
        self.inner_radius = inner_radius
        self.outer_radius = outer_radius
        self.smoothness = smoothness

    def __call__(self, *, r, **kwargs):
        return np.where(
            np.greater_equal(r, self.inner_radius) * np.less(r, self.outer_radius),
            np.abs(
                np.cos(0.5 * u.pi * (r - self.inner_radius) / np.abs(self.outer_radius - self.inner_radius))
            )
            ** (1 / self.smoothness),
            np.where(np.greater_equal(r, self.outer_radius), 0, 1),
        )

    def __repr__(self):
        return (
            f"{self.__class__.__name__}(inner_radius = {self.inner_radius}, "
            f"outer_radius = {self.outer_radius}, smoothness = {self.smoothness})"
        )


class AbsoluteRadialCosineMask(RadialCosineMask):
    """RadialCosineMask evaluated at |r|: on a line mesh it absorbs at both
    ends.  No counterpart class in the reference; it is the user ``Mask``
    subclass the two-sided 1D workload needs."""

    def __call__(self, *, r, **kwargs):
        return super().__call__(r=np.abs(r))
