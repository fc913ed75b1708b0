"""Atomic units: hbar = m_e = e = a_0 = 1/(4 pi eps_0) = 1.

The reference expresses everything in SI through ``simulacra.units``; this
package computes in atomic units throughout.  The constants below are the
ones the mesh path needs (CODATA 2018 values for the conversions).
"""

import math as _math

pi = _math.pi
twopi = 2 * _math.pi

hbar = 1.0
electron_mass = 1.0
electron_charge = -1.0
proton_charge = 1.0
bohr_radius = 1.0
per_bohr_radius = 1.0
hartree = 1.0
rydberg = 0.5
atomic_electric_field = 1.0
atomic_time = 1.0
coulomb_constant = 1.0
epsilon_0 = 1.0 / (4 * _math.pi)
c = 137.035999084
proton_mass = 1836.15267343
electron_mass_reduced = proton_mass * electron_mass / (proton_mass + electron_mass)

_bohr_m = 5.29177210903e-11
_atomic_time_s = 2.4188843265857e-17
_hartree_J = 4.3597447222071e-18
m = 1.0 / _bohr_m
nm = 1e-9 * m
s = 1.0 / _atomic_time_s
asec = 1e-18 * s
fsec = 1e-15 * s
eV = 1.602176634e-19 / _hartree_J
