"""ORACLE — host FP64 physics formulas restated from the reference (numpy).

Atomic units: hbar = m_e = e = a_0 = 1/(4 pi eps_0) = 1.  The electron charge
is -1 and the reduced electron mass uses m_p = 1836.15267343 m_e, the values
the golden fixtures were generated with.
"""

import math

import numpy as np
import scipy.special as special

HBAR = 1.0
ELECTRON_MASS = 1.0
ELECTRON_CHARGE = -1.0
PROTON_CHARGE = 1.0
BOHR_RADIUS = 1.0
COULOMB_CONSTANT = 1.0
PROTON_MASS = 1836.15267343
ELECTRON_MASS_REDUCED = PROTON_MASS * ELECTRON_MASS / (PROTON_MASS + ELECTRON_MASS)
SPEED_OF_LIGHT = 137.035999084
TWOPI = 2 * math.pi


class CosSquaredPulse:
    """E(t) of ionization/potentials/pulses.py:1696-1814 (CosSquaredPulse),
    built with ``from_omega_carrier`` (pulses.py:1716-1737)."""

    def __init__(self, amplitude, omega_carrier, number_of_cycles, phase=0.0, pulse_center=0.0):
        # from_omega_carrier stores a wavelength; omega is re-derived from it
        self.wavelength_carrier = SPEED_OF_LIGHT / (omega_carrier / TWOPI)
        self.amplitude = amplitude
        self.number_of_cycles = number_of_cycles
        self.phase = phase
        self.pulse_center = pulse_center

    @property
    def omega_carrier(self):
        return TWOPI * SPEED_OF_LIGHT / self.wavelength_carrier

    @property
    def period_carrier(self):
        return 1 / (SPEED_OF_LIGHT / self.wavelength_carrier)

    @property
    def total_time(self):
        return self.period_carrier * self.number_of_cycles

    def field(self, t):
        """pulses.py:1798-1814 (envelope then carrier, times amplitude)."""
        t = np.asarray(t, dtype=np.float64)
        tau = t - self.pulse_center
        env = np.where(
            np.less_equal(-self.total_time / 2, tau) * np.less_equal(tau, self.total_time / 2),
            np.cos(self.omega_carrier * tau / (2 * self.number_of_cycles)) ** 2,
            0,
        )
        amp = env * np.cos((self.omega_carrier * tau) + self.phase)
        return amp * self.amplitude * 1


def soft_coulomb(r, softening_distance, charge=PROTON_CHARGE, test_charge=ELECTRON_CHARGE):
    """potentials/static.py:75-91."""
    return COULOMB_CONSTANT * charge * test_charge / np.sqrt((r ** 2) + (softening_distance ** 2))


def coulomb(r, charge=PROTON_CHARGE, test_charge=ELECTRON_CHARGE):
    """potentials/static.py:26-38."""
    return COULOMB_CONSTANT * charge * test_charge / r


def radial_cosine_mask(r, inner_radius, outer_radius, smoothness):
    """potentials/masks.py:76-89."""
    return np.where(
        np.greater_equal(r, inner_radius) * np.less(r, outer_radius),
        np.abs(np.cos(0.5 * math.pi * (r - inner_radius) / np.abs(outer_radius - inner_radius)))
        ** (1 / smoothness),
        np.where(np.greater_equal(r, outer_radius), 0, 1),
    )


def hydrogen_radial(n, l, r, amplitude=1):
    """HydrogenBoundState.radial_function, states/three_d.py:375-391."""
    normalization = np.sqrt(
        ((2 / (n * BOHR_RADIUS)) ** 3)
        * (special.factorial(n - l - 1) / (2 * n * special.factorial(n + l)))
    )
    r_dep = np.exp(-r / (n * BOHR_RADIUS)) * ((2 * r / (n * BOHR_RADIUS)) ** l)
    lag_poly = special.eval_genlaguerre(n - l - 1, (2 * l) + 1, 2 * r / (n * BOHR_RADIUS))
    return amplitude * normalization * r_dep * lag_poly


def spherical_harmonic(l, m, theta, phi):
    return special.sph_harm_y(l, m, theta, phi)


def gaussian(z, width=1.0, center=0.0):
    return np.exp(-((z - center) ** 2) / (2 * width ** 2)).astype(np.complex128)
