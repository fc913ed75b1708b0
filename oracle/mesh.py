"""ORACLE — numpy restatement of the reference's mesh time-evolution path.

Every builder below mirrors one reference function (file:line in its
docstring) and keeps the reference's data layout: operators are the three
diagonals of a tridiagonal matrix over the mesh flattened in the operator's
wrapping order ("C" or "F", ionization/mesh/meshes.py:117-133), explicit
halves are a dia-matrix product (mesh_operators.py:104-106) and implicit
halves the Thomas solve of ``tdma.c`` on the whole flattened vector
(mesh_operators.py:109-111), exactly as the reference calls ``cy.tdma``.

Used only by tests/, smoke() and bench.py's CPU-baseline legs.
"""

import math

import numpy as np

from . import physics as ph
from ._lib import tdma


# --------------------------------------------------------------------------
# generic pieces
# --------------------------------------------------------------------------

def get_times(time_initial, time_final, time_step):
    """MeshSimulation.get_times, ionization/mesh/sims.py:198-205."""
    total_time = time_final - time_initial
    return np.linspace(time_initial, time_final, int(total_time / time_step) + 1)


def data_mask(n_times, store_data_every):
    """MeshSimulation.__init__ data mask, sims.py:84-90."""
    idx = np.arange(n_times)
    mask = np.equal(idx, 0) + np.equal(idx, n_times - 1)
    if store_data_every >= 1:
        mask += np.equal(idx % store_data_every, 0)
    return mask


class Tridiag:
    """A tridiagonal operator over a flattened mesh.

    ``sub[i]`` = A[i+1, i], ``diag[i]`` = A[i, i], ``sup[i]`` = A[i, i+1];
    ``order`` is the numpy flatten order of its wrapping direction (None for
    1D meshes)."""

    def __init__(self, sub, diag, sup, order):
        self.sub, self.diag, self.sup, self.order = sub, diag, sup, order

    def scaled_plus_identity(self, scale):
        """add_to_diagonal_sparse_matrix_diagonal(scale * M, value=1),
        mesh_operators.py:30-35 with evolution_methods.py:57-74."""
        return Tridiag(scale * self.sub, (scale * self.diag) + 1, scale * self.sup, self.order)


def dia_matvec(op: Tridiag, x):
    """y = A x accumulated diagonal by diagonal in the dia_matrix storage order
    (offsets -1, 0, +1), as DotOperator._apply (mesh_operators.py:104-106)."""
    y = np.zeros_like(x)
    y[1:] += op.sub * x[:-1]
    y += op.diag * x
    y[:-1] += op.sup * x[1:]
    return y


def _flat(g2d, order):
    return g2d if order is None else g2d.flatten(order)


def _wrap(vec, shape, order):
    return vec if order is None else np.reshape(vec, shape, order)


def apply_explicit(op, g, shape):
    return _wrap(dia_matvec(op, _flat(g, op.order)), shape, op.order)


def apply_implicit(op, g, shape):
    return _wrap(tdma(op.sub, op.diag, op.sup, _flat(g, op.order)), shape, op.order)


def run(stepper, times, store_data_every, max_steps=None, observe=None):
    """The data/evolve skeleton of MeshSimulation.run, sims.py:289-333.

    ``stepper`` exposes ``evolve(dt, t_now)``, ``norm()`` and
    ``inner_products()``.  Returns data-time norms and inner products, and
    ``observe(stepper)`` at each data time under "observed" when given."""
    mask = data_mask(len(times), store_data_every)
    norms, ips, dtimes, obs = [], [], [], []
    time_index = 0
    steps = 0
    while True:
        if mask[time_index]:
            norms.append(stepper.norm())
            ips.append(stepper.inner_products())
            dtimes.append(times[time_index])
            if observe is not None:
                obs.append(observe(stepper))
        if time_index == len(times) - 1:
            break
        if max_steps is not None and steps >= max_steps:
            break
        time_index += 1
        stepper.evolve(times[time_index] - times[time_index - 1], times[time_index])
        steps += 1
    return dict(
        data_times=np.array(dtimes),
        norm=np.array(norms),
        inner_products=np.array(ips).T if ips else np.zeros((0, 0)),
        steps=steps,
        observed=obs,
    )


# --------------------------------------------------------------------------
# position expectation values and partial norms
# --------------------------------------------------------------------------

def observables(stepper, kind, radii):
    """<z>, <r>, the norm within each radius and (SH) the norm of each l of the
    stepper's current g:
      QuantumMesh.expectation_value with the mesh's z / r operator
        (meshes.py:206-237): element-wise z_mesh, r_mesh on line and cylinder
        meshes (mesh_operators.py:344-349, 634-639); on the SH mesh z is the
        F-order off-diagonal c_l r operator (mesh_operators.py:1086-1104);
      NormWithinRadius.store: norm of where(r_mesh <= R, g, 0) (data.py:420-425);
      SphericalHarmonicMesh.norm_by_l (meshes.py:1133-1136)."""
    g = stepper.g
    p = (np.conj(g) * g).real
    if kind == "line":
        w, zw, rw = stepper.dz, stepper.z, stepper.z  # a line's r_mesh is z
        within = [np.sum(np.where(stepper.z <= R, p, 0.0)) * w for R in radii]
        return dict(z=np.sum(zw * p) * w, r=np.sum(rw * p) * w, within=within)
    if kind == "cyl":
        w = stepper.dz * stepper.drho
        within = [np.sum(np.where(stepper.r_mesh <= R, p, 0.0)) * w for R in radii]
        return dict(z=np.sum(stepper.z_mesh * p) * w, r=np.sum(stepper.r_mesh * p) * w, within=within)
    if kind == "sh":
        w = stepper.dr
        r = stepper.r[None, :]
        cl = np.array([_c_l(l) for l in range(stepper.L - 1)])[:, None]
        z = np.sum(2 * (np.conj(g[:-1]) * g[1:]).real * cl * r) * w
        within = [np.sum(np.where(stepper.r_mesh <= R, p, 0.0)) * w for R in radii]
        return dict(z=z, r=np.sum(p * r) * w, within=within, by_l=np.sum(p, axis=1) * w)
    raise ValueError(kind)


# --------------------------------------------------------------------------
# line mesh (LineMesh + LineLengthGaugeOperators)
# --------------------------------------------------------------------------

class LineLength:
    """LineMesh (meshes.py:263-341) with LineLengthGaugeOperators
    (mesh_operators.py:304-341); ``method`` is "AlternatingDirectionImplicit"
    (evolution_methods.py:46-77), "SplitInteractionOperator"
    (evolution_methods.py:80-123) or "FourierSplitOperator" (a numpy.fft
    statement of the Fourier split-step, which has no reference code).  The mask is RadialCosineMask evaluated at
    |z| (both line ends), and the initial state a Gaussian normalised on the
    mesh."""

    def __init__(self, z_points, z_bound, test_mass, softening_distance, pulse, mask, method,
                 gaussian_width=1.0, gauge="length"):
        self.gauge = gauge
        self.times = None  # the time grid, for the velocity gauge's vector potential
        self._index = 0
        self.z = np.linspace(-z_bound, z_bound, z_points)
        self.dz = np.abs(self.z[1] - self.z[0])
        self.shape = (z_points,)
        self.test_mass = test_mass
        self.pulse = pulse
        self.method = method
        self.mask = (
            ph.radial_cosine_mask(np.abs(self.z), **mask) if mask is not None else None
        )
        p = -(ph.HBAR ** 2) / (2 * test_mass * (self.dz ** 2))
        diag = -2 * p * np.ones(z_points, dtype=np.complex128)
        off = p * np.ones(z_points - 1, dtype=np.complex128)
        V = ph.soft_coulomb(self.z, softening_distance)
        self.V = np.asarray(V, dtype=np.float64)
        self.H0 = Tridiag(off, diag + 1.0 * V, off.copy(), None)  # mesh_operators.py:244-269
        k = 2 * np.pi * np.fft.fftfreq(z_points, d=self.dz)
        self.kin = (ph.HBAR ** 2) * k ** 2 / (2 * test_mass)
        g = ph.gaussian(self.z, gaussian_width)
        g = g / np.sqrt(self._norm(g))
        self.g = g
        self.test_g = [g.copy()]

    def _norm(self, g):
        return (np.sum(np.conj(g) * g) * self.dz).real

    def norm(self):
        return self._norm(self.g)

    def inner_products(self):
        return [np.sum(np.conj(s) * self.g) * self.dz for s in self.test_g]

    def v_int(self, t):
        """UniformLinearlyPolarizedElectricPotential.__call__, pulses.py:37-56."""
        return -self.z * ph.ELECTRON_CHARGE * self.pulse.field(t)

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        vint = self.v_int(t_now)  # mesh.sim.time is already t_{n+1}
        g = self.g
        if self.method == "FourierSplitOperator":
            # Fourier split-step (no reference counterpart): Strang splitting with
            # the kinetic factor applied exactly on the discrete Fourier modes
            p = np.exp(-1j * tau * (self.V + vint))
            g = p * g
            g = np.fft.ifft(np.exp(-1j * (2 * tau) * self.kin) * np.fft.fft(g))
            g = p * g
        elif self.gauge == "velocity":
            # LineVelocityGaugeOperators (mesh_operators.py:352-427) with
            # SplitInteractionOperator: S = (even, odd) real pair rotations
            self._index += 1
            A = vector_potential(self.pulse, self.times[: self._index + 1])
            off = ph.HBAR * (ph.ELECTRON_CHARGE / self.test_mass) / (2 * self.dz) * np.ones(len(self.z) - 1)
            even, odd = pair_rotations(tau * A * off, len(self.z) % 2 != 0, "velocity", None)
            g = apply_explicit(even, g, self.shape)
            g = apply_explicit(odd, g, self.shape)
            g = apply_explicit(self.H0.scaled_plus_identity(-1j * tau), g, self.shape)
            g = apply_implicit(self.H0.scaled_plus_identity(1j * tau), g, self.shape)
            g = apply_explicit(odd, g, self.shape)
            g = apply_explicit(even, g, self.shape)
        elif self.method == "AlternatingDirectionImplicit":
            H = Tridiag(self.H0.sub, self.H0.diag + 1.0 * vint, self.H0.sup, None)
            g = apply_explicit(H.scaled_plus_identity(-1j * tau), g, self.shape)
            g = apply_implicit(H.scaled_plus_identity(1j * tau), g, self.shape)
        else:
            s = np.exp(-1j * vint * tau)  # mesh_operators.py:329-341
            g = s * g
            g = apply_explicit(self.H0.scaled_plus_identity(-1j * tau), g, self.shape)
            g = apply_implicit(self.H0.scaled_plus_identity(1j * tau), g, self.shape)
            g = s * g
        if self.mask is not None:
            g = g * self.mask  # meshes.py:256-257
        self.g = g


# --------------------------------------------------------------------------
# spherical-harmonic mesh, length gauge, split-interaction operator
# --------------------------------------------------------------------------

def vector_potential(pulse, times):
    """ElectricPotential.get_vector_potential_amplitude_numeric at times[-1]
    (pulses.py:58-77): minus the Simpson integral of E over ``times`` (the
    reference's ``integrate.simps`` is scipy's ``simpson``)."""
    from scipy import integrate

    return -integrate.simpson(y=np.asarray(pulse.field(times), dtype=np.float64), x=times)


def pair_rotations(a, both_odd, gauge, order):
    """The even and odd operators of a split interaction over a flattened
    mesh with angles a[k] (pair (k, k+1)): mesh_operators.py:1037-1080
    (length gauge, [[cos, -i sin], [-i sin, cos]]), :1234-1268 and :385-424
    (velocity gauge, [[cos, sin], [-sin, cos]]).  ``both_odd``: the padding
    branch (an odd number of points), where the even operator leaves the last
    point alone and the odd one the first."""
    a_even, a_odd = a[::2], a[1::2]
    n = len(a) + 1
    even_diag = np.zeros(n, dtype=np.complex128)
    even_off = np.zeros(n - 1, dtype=np.complex128)
    odd_diag = np.zeros(n, dtype=np.complex128)
    odd_off = np.zeros(n - 1, dtype=np.complex128)
    sin = (lambda x: -1j * np.sin(x)) if gauge == "length" else np.sin
    if both_odd:
        even_diag[:-1] = np.cos(a_even).repeat(2)
        even_diag[-1] = 1
        even_off[::2] = sin(a_even)
        odd_diag[0] = 1
        odd_diag[1:] = np.cos(a_odd).repeat(2)
        odd_off[1::2] = sin(a_odd)
    else:
        even_diag[:] = np.cos(a_even).repeat(2)
        even_off[::2] = sin(a_even)
        odd_diag[0] = odd_diag[-1] = 1
        odd_diag[1:-1] = np.cos(a_odd).repeat(2)
        odd_off[1::2] = sin(a_odd)
    if gauge == "length":  # symmetric
        return Tridiag(even_off, even_diag, even_off, order), Tridiag(odd_off, odd_diag, odd_off, order)
    # antisymmetric: diags((-off, diag, off), offsets=(-1, 0, 1))
    return Tridiag(-even_off, even_diag, even_off, order), Tridiag(-odd_off, odd_diag, odd_off, order)


def _alpha(j):
    x = (j ** 2) + (2 * j)
    return (x + 1) / (x + 0.75)


def _beta(j):
    x = 2 * (j ** 2) + (2 * j)
    return (x + 1) / (x + 0.5)


def _c_l(l):
    return (l + 1) / np.sqrt(((2 * l) + 1) * ((2 * l) + 3))


class SphericalHarmonicSplit:
    """SphericalHarmonicMesh (meshes.py:985-1136) with
    SphericalHarmonicLengthGaugeOperators (mesh_operators.py:815-1080,
    Lagrangian kinetic energy with the hydrogen l=0 correction) and
    SplitInteractionOperator (evolution_methods.py:80-123)."""

    def __init__(self, r_points, r_bound, l_bound, pulse, mask, test_states, time_step,
                 initial_state=(1, 0)):
        r = np.linspace(0, r_bound, r_points)
        self.dr = r[1] - r[0]
        self.r = r + self.dr / 2
        self.Nr, self.L = r_points, l_bound
        self.shape = (l_bound, r_points)
        self.M = r_points * l_bound
        self.pulse = pulse
        self.time_step = time_step
        l_mesh, r_mesh = np.meshgrid(np.arange(l_bound), self.r, indexing="ij")
        self.r_mesh = r_mesh
        self.mask = ph.radial_cosine_mask(r_mesh, **mask) if mask is not None else None

        # kinetic_energy_from_lagrangian, mesh_operators.py:889-928
        mu = ph.ELECTRON_MASS_REDUCED
        p = -(ph.HBAR ** 2) / (2 * mu * (self.dr ** 2))
        k = np.arange(self.M)
        j = k % r_points
        diag = _beta(j).astype(np.complex128)
        dr_au = self.dr / ph.BOHR_RADIUS
        diag[0] += dr_au * (1 + dr_au) / 8
        kk = np.arange(self.M - 1)
        off = np.where((kk + 1) % r_points != 0, _alpha(kk % r_points), 0).astype(np.complex128)
        diag *= -2 * p
        off *= p
        eff = ((ph.HBAR ** 2) / (2 * mu)) * l_mesh * (l_mesh + 1) / (r_mesh ** 2)
        diag += eff.flatten("C")
        V = ph.coulomb(r_mesh)
        self.H0 = Tridiag(off, diag + 1.0 * V.flatten("C"), off.copy(), "C")

        # interaction_hamiltonian_matrices_without_field, mesh_operators.py:988-1005
        l_prefactor = -ph.ELECTRON_CHARGE * r_mesh.flatten("F")[:-1]
        l_off = np.where(
            (kk + 1) % l_bound != 0, _c_l(kk % l_bound), 0
        ).astype(np.complex128)
        l_off *= l_prefactor
        self.l_off = l_off

        self.test_states = list(test_states)
        self.radial_g = {}
        for (n, l) in self.test_states + [tuple(initial_state)]:
            gs = ph.hydrogen_radial(n, l, self.r) * self.r
            gs = gs / np.sqrt((np.sum(np.conj(gs) * gs) * self.dr).real)
            self.radial_g[(n, l)] = gs
        g = np.zeros(self.shape, dtype=np.complex128)
        n0, l0 = initial_state
        g[l0, :] += self.radial_g[(n0, l0)]
        self.g = g
        self._cn_cache = {}

    def norm(self):
        return (np.sum(np.conj(self.g) * self.g) * self.dr).real

    def inner_products(self):
        """SphericalHarmonicMesh.inner_product shortcut, meshes.py:1118-1129."""
        return [
            (0 + np.sum(np.conj(self.radial_g[(n, l)]) * self.g[l, :])) * self.dr
            for (n, l) in self.test_states
        ]

    def split_operators(self, tau, efield):
        """split_interaction_operators, mesh_operators.py:1037-1080."""
        a = tau * (self.l_off * efield)
        return pair_rotations(a, self.Nr % 2 != 0 and self.L % 2 != 0, "length", "F")

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        efield = self.pulse.field(t_now + (self.time_step / 2))  # mesh_operators.py:1011-1013
        even, odd = self.split_operators(tau, efield)
        g = self.g
        g = apply_explicit(even, g, self.shape)
        g = apply_explicit(odd, g, self.shape)
        g = apply_explicit(self.H0.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(self.H0.scaled_plus_identity(1j * tau), g, self.shape)
        g = apply_explicit(odd, g, self.shape)
        g = apply_explicit(even, g, self.shape)
        if self.mask is not None:
            g = g * self.mask
        self.g = g


class SphericalHarmonicADI(SphericalHarmonicSplit):
    """SphericalHarmonicMesh with SphericalHarmonicLengthGaugeOperators and
    AlternatingDirectionImplicit (evolution_methods.py:46-77): the operators of
    total_hamiltonian (mesh_operators.py:1020-1035) are the radial H0 ("r",
    C order) and the l-coupling interaction ("l", F order, field at
    t + time_step / 2), taken explicit, implicit, explicit, implicit over
    [H0, H_int, H_int, H0]; then the mask."""

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        efield = self.pulse.field(t_now + (self.time_step / 2))
        off = self.l_off * efield
        hint = Tridiag(off, np.zeros(self.M, dtype=np.complex128), off.copy(), "F")
        g = self.g
        g = apply_explicit(self.H0.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(hint.scaled_plus_identity(1j * tau), g, self.shape)
        g = apply_explicit(hint.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(self.H0.scaled_plus_identity(1j * tau), g, self.shape)
        if self.mask is not None:
            g = g * self.mask
        self.g = g


class SphericalHarmonicVelocity(SphericalHarmonicSplit):
    """SphericalHarmonicMesh with SphericalHarmonicVelocityGaugeOperators
    (mesh_operators.py:1130-1408) and SplitInteractionOperator: per step
    S = (h1 even, h1 odd, h2 even-even, even-odd, odd-even, odd-odd), the
    radial Crank-Nicolson pair, reversed S, the mask.  The field enters as the
    vector potential at the current time (times_to_current, sims.py:195-196)."""

    def __init__(self, *args, test_mass=ph.ELECTRON_MASS_REDUCED, **kw):
        super().__init__(*args, **kw)
        self.times = None
        self._index = 0
        q_over_m = ph.ELECTRON_CHARGE / test_mass
        kk = np.arange(self.M - 1)
        l_of = kk % self.L
        r_f = self.r_mesh.flatten("F")[:-1]
        # h1 (mesh_operators.py:1143-1158) without i and the field:
        # hbar (q/m) c_l (l+1) / r on F-order neighbours of one r
        self.h1_off = np.where((kk + 1) % self.L != 0, _c_l(l_of) * (l_of + 1), 0.0) * (ph.HBAR * q_over_m) / r_f
        # h2 = hbar (q/m) / (2 dr) kron(c_block, alpha_block) (:1160-1176)
        self.h2_l = _c_l(np.arange(self.L - 1))
        self.h2_r = (ph.HBAR * q_over_m / (2 * self.dr)) * _alpha(np.arange(self.Nr - 1))

    def _similarity(self, g, parity):
        """SimilarityOperator.u_even_g / u_odd_g (mesh_operators.py:166-189)
        along l: rows (l, l+1) of each pair -> ((a + b), (a - b)) / sqrt 2, the
        unpaired rows as sqrt(2) g / sqrt(2)."""
        s2 = np.sqrt(2)
        out = (s2 * g) / s2
        first = np.arange(parity, self.L - 1, 2)
        a, b = g[first], g[first + 1]
        out[first] = (a + b) / s2
        out[first + 1] = (a - b) / s2
        return out

    def _h2(self, g, tau, A, lpar, rpar):
        """One SimilarityOperator of split_h2 (mesh_operators.py:1270-1408):
        in the transformed rows of l-pair (l, l+1) the r-pairs (r, r+1) of
        parity ``rpar`` turn by [[cos, sin], [-sin, cos]] with angle
        tau A c_l alpha(r) hbar (q/m) / (2 dr), the (a - b) row by the
        opposite angle; then the transform back."""
        u = self._similarity(g, lpar)
        first = np.arange(lpar, self.L - 1, 2)
        rs = np.arange(rpar, self.Nr - 1, 2)
        th = tau * A * self.h2_l[first][:, None] * self.h2_r[rs][None, :]
        c, s = np.cos(th), np.sin(th)
        for row, sign in ((first, 1.0), (first + 1, -1.0)):
            x0, x1 = u[row][:, rs], u[row][:, rs + 1]
            y0 = c * x0 + (sign * s) * x1
            y1 = -(sign * s) * x0 + c * x1
            blk = u[row]
            blk[:, rs], blk[:, rs + 1] = y0, y1
            u[row] = blk
        return self._similarity(u, lpar)

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        self._index += 1
        A = vector_potential(self.pulse, self.times[: self._index + 1])
        h1e, h1o = pair_rotations(tau * A * self.h1_off, self.Nr % 2 != 0 and self.L % 2 != 0, "velocity", "F")
        g = self.g
        g = apply_explicit(h1e, g, self.shape)
        g = apply_explicit(h1o, g, self.shape)
        for lp, rp in ((0, 0), (0, 1), (1, 0), (1, 1)):
            g = self._h2(g, tau, A, lp, rp)
        g = apply_explicit(self.H0.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(self.H0.scaled_plus_identity(1j * tau), g, self.shape)
        for lp, rp in ((1, 1), (1, 0), (0, 1), (0, 0)):
            g = self._h2(g, tau, A, lp, rp)
        g = apply_explicit(h1o, g, self.shape)
        g = apply_explicit(h1e, g, self.shape)
        if self.mask is not None:
            g = g * self.mask
        self.g = g


# --------------------------------------------------------------------------
# cylindrical slice mesh, length gauge, ADI
# --------------------------------------------------------------------------

class CylindricalSliceADI:
    """CylindricalSliceMesh (meshes.py:509-607) with
    CylindricalSliceLengthGaugeOperators (mesh_operators.py:550-640) and
    AlternatingDirectionImplicit (evolution_methods.py:46-77)."""

    def __init__(self, z_points, z_bound, rho_points, rho_bound, pulse, test_states,
                 test_mass=ph.ELECTRON_MASS_REDUCED, initial_state=(1, 0)):
        self.z = np.linspace(-z_bound, z_bound, z_points)
        rho = np.delete(np.linspace(0, rho_bound, rho_points + 1), 0)
        self.dz = self.z[1] - self.z[0]
        self.drho = rho[1] - rho[0]
        self.rho = rho - self.drho / 2
        self.shape = (z_points, rho_points)
        self.Nz, self.Nrho = z_points, rho_points
        self.M = z_points * rho_points
        self.pulse = pulse
        self.z_mesh, self.rho_mesh = np.meshgrid(self.z, self.rho, indexing="ij")
        self.r_mesh = np.sqrt((self.z_mesh ** 2) + (self.rho_mesh ** 2))
        self.theta_mesh = np.arccos(self.z_mesh / self.r_mesh)
        self.g_factor = np.sqrt(ph.TWOPI * self.rho_mesh)
        self.mult = self.dz * self.drho

        M = self.M
        kk = np.arange(M - 1)
        pz = -(ph.HBAR ** 2) / (2 * test_mass * (self.dz ** 2))
        z_diag = pz * (-2) * np.ones(M, dtype=np.complex128)
        z_off = pz * np.where((kk + 1) % z_points != 0, 1, 0).astype(np.complex128)
        prho = -(ph.HBAR ** 2) / (2 * test_mass * (self.drho ** 2))
        rho_diag = prho * (-2) * np.ones(M, dtype=np.complex128)
        jj = (kk % rho_points) + 1
        cj = jj / np.sqrt((jj ** 2) - 0.25)
        rho_off = np.where((kk + 1) % rho_points != 0, cj, 0).astype(np.complex128)
        rho_off *= prho
        V = ph.coulomb(self.r_mesh)
        pre = 1 / 2
        # internal_hamiltonian, mesh_operators.py:244-269 (order: rho, z)
        self.H_rho0 = Tridiag(rho_off, rho_diag + pre * V.flatten("C"), rho_off.copy(), "C")
        self.H_z0 = Tridiag(z_off, z_diag + pre * V.flatten("F"), z_off.copy(), "F")

        self.test_states = list(test_states)
        self.test_g = {}
        for (n, l) in self.test_states + [tuple(initial_state)]:
            self.test_g[(n, l)] = self._state_g(n, l)
        self.g = self.test_g[tuple(initial_state)].copy()

    def _state_g(self, n, l):
        """CylindricalSliceMesh.get_g_for_state, meshes.py:601-607."""
        psi = 1 * ph.hydrogen_radial(n, l, self.r_mesh) * ph.spherical_harmonic(
            l, 0, self.theta_mesh, 0
        )
        g = self.g_factor * psi
        g = g / np.sqrt((np.sum(np.conj(g) * g) * self.mult).real)
        return g

    def norm(self):
        return (np.sum(np.conj(self.g) * self.g) * self.mult).real

    def inner_products(self):
        return [np.sum(np.conj(self.test_g[s]) * self.g) * self.mult for s in self.test_states]

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        epot = -self.z_mesh * ph.ELECTRON_CHARGE * self.pulse.field(t_now)
        pre = 1 / 2
        # total_hamiltonian, mesh_operators.py:271-298
        H_rho = Tridiag(self.H_rho0.sub, self.H_rho0.diag + pre * epot.flatten("C"), self.H_rho0.sup, "C")
        H_z = Tridiag(self.H_z0.sub, self.H_z0.diag + pre * epot.flatten("F"), self.H_z0.sup, "F")
        g = self.g
        g = apply_explicit(H_rho.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(H_z.scaled_plus_identity(1j * tau), g, self.shape)
        g = apply_explicit(H_z.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(H_rho.scaled_plus_identity(1j * tau), g, self.shape)
        self.g = g


# --------------------------------------------------------------------------
# builders from fixture parameter dicts
# --------------------------------------------------------------------------

# --------------------------------------------------------------------------
# rectangle mesh, length gauge, ADI
# --------------------------------------------------------------------------

class RectangleADI:
    """RectangleMesh (meshes.py:430-506) with RectangleLengthGaugeOperators
    (mesh_operators.py:430-505) and AlternatingDirectionImplicit
    (evolution_methods.py:46-77): kinetic energies along z ("z", F order) and
    x ("x", C order), in that order, each with half the internal potential
    (mesh_operators.py:244-269) and half of -z q E(t_{n+1})
    (mesh_operators.py:271-298); steps E(H_z), I(H_x), E(H_x), I(H_z), then
    the mask.  The initial state is TwoDGaussianWavepacket (states/two_d.py:
    259-315) evaluated through (r, theta = arctan2(x, z)) as
    RectangleMesh.get_g_for_state does."""

    def __init__(self, z_points, z_bound, x_points, x_bound, softening_distance, pulse, mask, state,
                 test_mass=ph.ELECTRON_MASS_REDUCED):
        self.z = np.linspace(-z_bound, z_bound, z_points)
        self.x = np.linspace(-x_bound, x_bound, x_points)
        self.dz, self.dx = abs(self.z[1] - self.z[0]), abs(self.x[1] - self.x[0])
        self.shape = (z_points, x_points)
        self.M = z_points * x_points
        self.pulse = pulse
        z_mesh, x_mesh = np.meshgrid(self.z, self.x, indexing="ij")
        self.z_mesh, self.x_mesh = z_mesh, x_mesh
        self.r_mesh = np.sqrt(z_mesh ** 2 + x_mesh ** 2)
        self.theta_mesh = np.arctan2(x_mesh, z_mesh)
        self.mask = ph.radial_cosine_mask(self.r_mesh, **mask) if mask is not None else None
        V = ph.soft_coulomb(self.r_mesh, softening_distance)
        self.H = []
        for n_dir, d, order in ((z_points, self.dz, "F"), (x_points, self.dx, "C")):
            p = -(ph.HBAR ** 2) / (2 * test_mass * d ** 2)
            diag = -2 * p * np.ones(self.M, dtype=np.complex128)
            kk = np.arange(self.M - 1)
            off = p * np.where((kk + 1) % n_dir != 0, 1.0, 0.0).astype(np.complex128)
            self.H.append(Tridiag(off, diag + 0.5 * V.flatten(order), off.copy(), order))
        self.zq = {o: (-ph.ELECTRON_CHARGE * z_mesh).flatten(o) for o in ("F", "C")}
        g = self._state(state)
        self.g = g
        self.test_g = [g.copy()]

    def _state(self, st):
        cz, cx, wz, wx, kz, kx = st
        z = self.r_mesh * np.cos(self.theta_mesh)
        x = self.r_mesh * np.sin(self.theta_mesh)
        norm = 1 / (np.sqrt(ph.TWOPI) * np.sqrt(wz * wx))
        g = norm * np.exp(-0.5 * (((z - cz) / wz) ** 2)) * np.exp(-0.5 * (((x - cx) / wx) ** 2)) \
            * (np.exp(1j * kz * z) * np.exp(1j * kx * x))
        return g / np.sqrt(self._norm(g))

    def _norm(self, g):
        return (np.sum(np.conj(g) * g) * self.dz * self.dx).real

    def norm(self):
        return self._norm(self.g)

    def inner_products(self):
        return [np.sum(np.conj(s) * self.g) * self.dz * self.dx for s in self.test_g]

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        E = self.pulse.field(t_now)
        ops = [Tridiag(h.sub, h.diag + 0.5 * self.zq[h.order] * E, h.sup, h.order) for h in self.H]
        hz, hx = ops
        g = self.g
        g = apply_explicit(hz.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(hx.scaled_plus_identity(1j * tau), g, self.shape)
        g = apply_explicit(hx.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(hz.scaled_plus_identity(1j * tau), g, self.shape)
        if self.mask is not None:
            g = g * self.mask
        self.g = g


# --------------------------------------------------------------------------
# spherical slice mesh, length gauge, ADI
# --------------------------------------------------------------------------

class SphericalSliceADI:
    """SphericalSliceMesh (meshes.py:887-983) with
    SphericalSliceLengthGaugeOperators (mesh_operators.py:693-813) and
    AlternatingDirectionImplicit: kinetic energies along theta ("theta",
    C order, a non-symmetric tridiagonal) and r ("r", F order), in that
    order, each with half of the Coulomb potential and half of -z q E(t_{n+1});
    steps E(H_theta), I(H_r), E(H_r), I(H_theta), then the mask.  g = g_factor
    psi with g_factor = sqrt(2 pi sin theta) r."""

    def __init__(self, r_points, r_bound, theta_points, pulse, mask, test_states, initial_state=(1, 0)):
        r = np.linspace(0, r_bound, r_points)
        th = np.delete(np.linspace(0, np.pi, theta_points + 1), 0)
        self.dr, self.dth = r[1] - r[0], th[1] - th[0]
        self.r, self.theta = r + self.dr / 2, th - self.dth / 2
        self.shape = (r_points, theta_points)
        self.M = r_points * theta_points
        self.pulse = pulse
        r_mesh, th_mesh = np.meshgrid(self.r, self.theta, indexing="ij")
        self.r_mesh, self.th_mesh = r_mesh, th_mesh
        self.z_mesh = r_mesh * np.cos(th_mesh)
        self.mask = ph.radial_cosine_mask(r_mesh, **mask) if mask is not None else None
        mu = ph.ELECTRON_MASS_REDUCED
        V = ph.coulomb(r_mesh)
        nth = theta_points
        # theta kinetic (mesh_operators.py:724-775), C order: index = j * nth + k
        pt = -(ph.HBAR ** 2) / (2 * mu * ((self.dr * self.dth) ** 2))
        idx = np.arange(self.M)
        jj = idx // nth
        tjp = lambda x: 1 / (x + 0.5) ** 2  # noqa: E731
        sink = lambda x: np.sin(x * self.dth)  # noqa: E731
        cotk = lambda x: 1 / np.tan(x * self.dth)  # noqa: E731
        tdiag = (-2) * tjp(jj) * pt
        kk = np.arange(self.M - 1)
        j1, k1 = kk // nth, kk % nth
        live = (kk + 1) % nth != 0
        kp = k1 + 1
        with np.errstate(invalid="ignore", divide="ignore"):  # the dead entries at block ends
            upper = np.where(live, tjp(j1) * (1 + (self.dth / 2) * cotk(k1 + 0.5)) * np.sqrt(sink(k1 + 0.5) / sink(k1 + 1.5)), 0) * pt
            lower = np.where(live, tjp(j1) * (1 - (self.dth / 2) * cotk(kp + 0.5)) * np.sqrt(sink(kp + 0.5) / sink(kp - 0.5)), 0) * pt
        self.Hth = Tridiag(lower.astype(np.complex128), (tdiag + 0.5 * V.flatten("C")).astype(np.complex128),
                           upper.astype(np.complex128), "C")
        # r kinetic (:704-722), F order: index = k * nr + j
        pr = -(ph.HBAR ** 2) / (2 * mu * (self.dr ** 2))
        roff = pr * np.where((kk + 1) % r_points != 0, 1.0, 0.0)
        self.Hr = Tridiag(roff.astype(np.complex128), (-2 * pr + 0.5 * V.flatten("F")).astype(np.complex128),
                          roff.astype(np.complex128), "F")
        self.zq = {o: (-ph.ELECTRON_CHARGE * self.z_mesh).flatten(o) for o in ("F", "C")}
        self.g_factor = np.sqrt(2 * np.pi * np.sin(th_mesh)) * r_mesh
        self.test_g = [self._state(n, l) for (n, l) in test_states]
        self.g = self._state(*initial_state)

    def _state(self, n, l):
        psi = ph.hydrogen_radial(n, l, self.r_mesh) * ph.spherical_harmonic(l, 0, self.th_mesh, 0)
        g = self.g_factor * psi
        return g / np.sqrt(self._norm(g))

    def _norm(self, g):
        return (np.sum(np.conj(g) * g) * self.dr * self.dth).real

    def norm(self):
        return self._norm(self.g)

    def inner_products(self):
        return [np.sum(np.conj(s) * self.g) * self.dr * self.dth for s in self.test_g]

    def evolve(self, dt, t_now):
        tau = dt / (2 * ph.HBAR)
        E = self.pulse.field(t_now)
        hth = Tridiag(self.Hth.sub, self.Hth.diag + 0.5 * self.zq["C"] * E, self.Hth.sup, "C")
        hr = Tridiag(self.Hr.sub, self.Hr.diag + 0.5 * self.zq["F"] * E, self.Hr.sup, "F")
        g = self.g
        g = apply_explicit(hth.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(hr.scaled_plus_identity(1j * tau), g, self.shape)
        g = apply_explicit(hr.scaled_plus_identity(-1j * tau), g, self.shape)
        g = apply_implicit(hth.scaled_plus_identity(1j * tau), g, self.shape)
        if self.mask is not None:
            g = g * self.mask
        self.g = g


# --------------------------------------------------------------------------
# numeric eigenstate basis
# --------------------------------------------------------------------------

def single_l_hamiltonian(r_points, r_bound, l):
    """internal_hamiltonian_for_single_l with the Lagrangian kinetic energy
    (mesh_operators.py:942-986): (diagonal, off-diagonal), real."""
    r = np.linspace(0, r_bound, r_points)
    dr = r[1] - r[0]
    r = r + dr / 2
    mu = ph.ELECTRON_MASS_REDUCED
    p = -(ph.HBAR ** 2) / (2 * mu * (dr ** 2))
    eff = ((ph.HBAR ** 2) / (2 * mu)) * l * (l + 1) / (r ** 2)
    beta = _beta(np.arange(r_points, dtype=np.complex128))
    if l == 0:
        d = dr / ph.BOHR_RADIUS
        beta[0] += d * (1 + d) / 8
    diag = (-2 * p * beta) + eff + ph.coulomb(r)
    off = p * _alpha(np.arange(r_points - 1, dtype=np.complex128))
    return diag.real, off.real, r, dr


def numeric_eigenbasis(r_points, r_bound, max_energy, max_l):
    """get_numeric_eigenstate_basis (meshes.py:1281-1356) with LAPACK's
    tridiagonal eigensolver in place of eigsh: per l, the eigenpairs with
    energy <= max_energy (at most r_points - 2, the smallest), each vector
    normalised on the mesh (dr sum |v|^2 = 1).  Returns [(l, energy, v)]
    sorted by energy; the vectors' signs are arbitrary."""
    from scipy.linalg import eigh_tridiagonal

    out = []
    for l in range(max_l + 1):
        d, e, r, dr = single_l_hamiltonian(r_points, r_bound, l)
        w, v = eigh_tridiagonal(d, e, select="v", select_range=(-np.inf, max_energy))
        w, v = w[: r_points - 2], v[:, : r_points - 2]
        for k in range(len(w)):
            vec = v[:, k] / np.sqrt(dr * np.sum(np.abs(v[:, k]) ** 2))
            out.append((l, w[k], vec))
    return sorted(out, key=lambda x: x[1])


def pulse_from_params(p):
    return ph.CosSquaredPulse(
        amplitude=p["amplitude"],
        omega_carrier=p["omega_carrier"],
        number_of_cycles=p["number_of_cycles"],
        phase=p["phase"],
        pulse_center=p["pulse_center"],
    )


def build_from_params(kind, params):
    pulse = pulse_from_params(params["pulse"])
    if kind == "line":
        method = params["method"]
        return LineLength(
            params["z_points"], params["z_bound"], params["test_mass"],
            params["softening_distance"], pulse, params.get("mask"), method,
            params.get("gaussian_width", 1.0), gauge=params.get("gauge", "length"),
        )
    if kind == "sh":
        cls = SphericalHarmonicVelocity if params.get("gauge", "length") == "velocity" else SphericalHarmonicSplit
        if params.get("method", "SplitInteractionOperator") == "AlternatingDirectionImplicit":
            cls = SphericalHarmonicADI
        return cls(
            params["r_points"], params["r_bound"], params["l_bound"], pulse, params.get("mask"),
            [tuple(s) for s in params["test_states"]], params["time_step"],
        )
    if kind == "slice":
        return SphericalSliceADI(
            params["r_points"], params["r_bound"], params["theta_points"], pulse, params.get("mask"),
            [tuple(x) for x in params["test_states"]],
        )
    if kind == "rect":
        st = (params["center_z"], params["center_x"], params["width_z"], params["width_x"], params["k_z"],
              params.get("k_x", 0.0))
        return RectangleADI(
            params["z_points"], params["z_bound"], params["x_points"], params["x_bound"],
            params["softening_distance"], pulse, params.get("mask"), st,
        )
    if kind == "cyl":
        return CylindricalSliceADI(
            params["z_points"], params["z_bound"], params["rho_points"], params["rho_bound"],
            pulse, [tuple(s) for s in params["test_states"]],
        )
    raise ValueError(kind)


def run_from_params(kind, params, max_steps=None, radii=None):
    stepper = build_from_params(kind, params)
    times = get_times(params["time_initial"], params["time_final"], params["time_step"])
    stepper.times = times
    g0 = stepper.g.copy()
    observe = None if radii is None else (lambda st: observables(st, kind, radii))
    out = run(stepper, times, params["store_data_every"], max_steps=max_steps, observe=observe)
    out["times"] = times
    out["g_initial"] = g0
    out["g_final"] = stepper.g
    out["stepper"] = stepper
    return out
