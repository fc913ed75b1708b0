"""Atomic units (hbar = m_e = e = a_0 = 1/(4 pi eps_0) = 1) for the reference stub.

Only the constants the mesh path uses carry physical meaning here; any other
name resolves to 1.0 through the module-level ``__getattr__`` so that the
reference's import-time defaults (e.g. ``800 * u.nm``) evaluate.
"""

import math as _math

pi = _math.pi
twopi = 2 * _math.pi

hbar = 1.0
electron_mass = 1.0
electron_charge = -1.0
proton_charge = 1.0
e = 1.0
bohr_radius = 1.0
per_bohr_radius = 1.0
hartree = 1.0
rydberg = 0.5
atomic_electric_field = 1.0
atomic_time = 1.0
atomic_force = 1.0
atomic_momentum = 1.0
atomic_electric_dipole_moment = 1.0
coulomb_constant = 1.0
epsilon_0 = 1.0 / (4 * _math.pi)
c = 137.035999084

proton_mass = 1836.15267343
electron_mass_reduced = proton_mass * electron_mass / (proton_mass + electron_mass)

# SI-derived units expressed in atomic units
_bohr_m = 5.29177210903e-11
_atomic_time_s = 2.4188843265857e-17
_hartree_J = 4.3597447222071e-18
m = 1.0 / _bohr_m
cm = 1e-2 * m
nm = 1e-9 * m
per_nm = 1.0 / nm
s = 1.0 / _atomic_time_s
asec = 1e-18 * s
fsec = 1e-15 * s
Hz = 1.0 / s
THz = 1e12 * Hz
J = 1.0 / _hartree_J
eV = 1.602176634e-19 * J
N = J / m
N_per_m = N / m
V_per_m = (J / 1.602176634e-19) / m  # volt = J/C, C = 1/e_SI in a.u. charge
W = J / s
TW = 1e12 * W
TWcm2 = TW / (cm ** 2)
Jcm2 = J / (cm ** 2)
deg = pi / 180


class Unit(float):
    pass


def get_unit_value_and_latex(unit):
    return 1.0, ""


def __getattr__(name):
    if name.startswith("__"):
        raise AttributeError(name)
    return 1.0
