"""``simulacra.math`` pieces used by the reference (stub)."""

import numpy as np
import scipy.special as special


class SphericalHarmonic:
    def __init__(self, l=0, m=0):
        self.l = int(l)
        self.m = int(m)

    def __hash__(self):
        return hash((self.__class__.__name__, self.l, self.m))

    def __eq__(self, other):
        return isinstance(other, SphericalHarmonic) and (self.l, self.m) == (
            other.l,
            other.m,
        )

    def __lt__(self, other):
        return (self.l, self.m) < (other.l, other.m)

    def __call__(self, theta, phi=0):
        return special.sph_harm_y(self.l, self.m, theta, phi)

    def __repr__(self):
        return f"SphericalHarmonic(l={self.l}, m={self.m})"


def complex_nquad(func, ranges, **kwargs):
    import scipy.integrate as integ

    re = integ.nquad(lambda *a: np.real(func(*a)), ranges, **kwargs)
    im = integ.nquad(lambda *a: np.imag(func(*a)), ranges, **kwargs)
    return re[0] + 1j * im[0], re[1:], im[1:]
