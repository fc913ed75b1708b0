"""Discretised Hamiltonians of the mesh path (host FP64 coefficient build).

The classes keep the reference's names and plug-in role
(ionization/mesh/mesh_operators.py:221-1128): a ``MeshOperators`` instance is
given to a specification and turns a mesh into operators.  Here their main
product is the set of FP64 coefficient tables the CUDA kernels consume
(``device_tables``); the tables are computed with the reference's formulas and
operation order so that the device sees bit-identical coefficients.  The
sparse-matrix views (``kinetic_energy``, ``internal_hamiltonian``, ...) are
kept for inspection and for host-side operator application.
"""

import numpy as np
import scipy.sparse as sparse

from .. import core
from .. import units as u


class SimilarityOperatorParity(core.StrEnum):
    EVEN = "even"
    ODD = "odd"


class KineticEnergyDerivation(core.StrEnum):
    HAMILTONIAN = "hamiltonian"
    LAGRANGIAN = "lagrangian"


def add_to_diagonal_sparse_matrix_diagonal(dia_matrix, value=1):
    """mesh_operators.py:30-35."""
    s = dia_matrix.copy()
    s.setdiag(s.diagonal() + value)
    return s


class MeshOperator:
    """A sparse tridiagonal operator with a wrapping direction
    (mesh_operators.py:45-93).  ``apply`` works on host arrays."""

    def __init__(self, matrix, *, wrapping_direction):
        self.matrix = matrix
        self.wrapping_direction = wrapping_direction

    def __repr__(self):
        return f"{self.__class__.__name__}(wrapping_direction = {self.wrapping_direction})"

    def apply(self, mesh, g, current_wrapping_direction):
        if current_wrapping_direction != self.wrapping_direction:
            g = mesh.flatten_mesh(mesh.wrap_vector(g, current_wrapping_direction), self.wrapping_direction)
        return self._apply(g), self.wrapping_direction

    def _apply(self, g):
        raise NotImplementedError


class DotOperator(MeshOperator):
    def _apply(self, g):
        return self.matrix.dot(g)


class TDMAOperator(MeshOperator):
    """Implicit half-step: solved by the GPU Thomas solver (the drop-in for
    ``cy.tdma``, mesh_operators.py:109-111)."""

    def _apply(self, g):
        from ..cy import tdma

        return tdma(self.matrix, g)


class SumOfOperators:
    def __init__(self, *operators):
        self.operators = tuple(operators)

    def apply(self, mesh, g, current_wrapping_direction):
        if len(self.operators) == 0:
            return g, current_wrapping_direction
        result = np.zeros_like(g)
        for operator in self.operators:
            r, wrapping = operator.apply(mesh, g, current_wrapping_direction)
            result += mesh.wrap_vector(r, wrapping)
        return result, current_wrapping_direction

    def __iter__(self):
        yield from self.operators

    def __getitem__(self, item):
        return self.operators[item]


def apply_operators_sequentially(mesh, g, operators):
    """mesh_operators.py:207-218 (host application)."""
    current = None
    for operator in operators:
        g, current = operator.apply(mesh, g, current)
    return mesh.wrap_vector(g, current)


class MeshOperators:
    gauge = None

    def __repr__(self):
        return f"{self.__class__.__name__}()"

    def info(self):
        return self.__class__.__name__


def _memo(method):
    """Per-(operators, mesh) memoisation, like si.utils.memoize on methods."""
    name = "_memo_" + method.__name__

    def wrapper(self, mesh, *args):
        cache = mesh.__dict__.setdefault(name, {})
        key = (id(self),) + args
        if key not in cache:
            cache[key] = method(self, mesh, *args)
        return cache[key]

    wrapper.__name__ = method.__name__
    wrapper.__doc__ = method.__doc__
    return wrapper


# --------------------------------------------------------------------------
# line mesh
# --------------------------------------------------------------------------


class LineLengthGaugeOperators(MeshOperators):
    """mesh_operators.py:304-341."""

    gauge = core.Gauge.LENGTH

    @_memo
    def device_tables(self, mesh):
        """(hd, hoff, zq): diagonal of H0 = kinetic + V (mesh_operators.py:309-318,
        244-269), its off-diagonal, and the interaction per unit field
        -z * test_charge (pulses.py:37-56)."""
        spec = mesh.spec
        prefactor = -(u.hbar ** 2) / (2 * spec.test_mass * (mesh.delta_z ** 2))
        diag = -2 * prefactor * np.ones(len(mesh.z_mesh), dtype=np.complex128)
        off = prefactor * np.ones(len(mesh.z_mesh) - 1, dtype=np.complex128)
        V = spec.internal_potential(r=mesh.r_mesh, z=mesh.z_mesh, test_charge=spec.test_charge)
        hd = (diag + 1.0 * V).real.copy()
        zq = -mesh.z_mesh * spec.test_charge
        return hd, off.real.copy(), np.asarray(zq, dtype=np.float64)

    @_memo
    def fourier_tables(self, mesh):
        """(V, kin, twiddle) for FourierSplitOperator: the static potential on
        the z mesh, the kinetic energy hbar^2 k^2 / (2 m) of each Fourier mode
        (k = 2 pi fftfreq(n, dz)) placed at the position the device's in-place
        transform leaves it (bit-reversed index), and exp(-2 pi i m / n)."""
        spec = mesh.spec
        n = len(mesh.z_mesh)
        if n < 2 or n & (n - 1):
            raise ValueError(f"FourierSplitOperator needs a power-of-two number of z points, not {n}")
        V = np.asarray(spec.internal_potential(r=mesh.r_mesh, z=mesh.z_mesh, test_charge=spec.test_charge))
        V = np.broadcast_to(V.real.astype(np.float64), (n,)).copy()
        k = 2 * np.pi * np.fft.fftfreq(n, d=mesh.delta_z)
        kin = (u.hbar ** 2) * (k ** 2) / (2 * spec.test_mass)
        bits = n.bit_length() - 1
        idx = np.arange(n)
        rev = np.zeros(n, dtype=np.int64)
        for b in range(bits):
            rev |= ((idx >> b) & 1) << (bits - 1 - b)
        twiddle = np.exp(-2j * np.pi * np.arange(n) / n)
        return V, kin[rev].copy(), twiddle

    @_memo
    def internal_hamiltonian(self, mesh):
        hd, hoff, _ = self.device_tables(mesh)
        m = sparse.diags((hoff.astype(np.complex128), hd.astype(np.complex128), hoff.astype(np.complex128)),
                         offsets=(-1, 0, 1))
        return SumOfOperators(DotOperator(m, wrapping_direction=None))

    def interaction_hamiltonian(self, mesh):
        epot = mesh.spec.electric_potential(t=mesh.sim.time, z=mesh.z_mesh, test_charge=mesh.spec.test_charge)
        return SumOfOperators(DotOperator(sparse.diags((epot,), offsets=(0,)), wrapping_direction=None))

    def total_hamiltonian(self, mesh):
        internal = self.internal_hamiltonian(mesh).operators[0]
        interaction = self.interaction_hamiltonian(mesh).operators[0]
        return SumOfOperators(
            DotOperator(
                add_to_diagonal_sparse_matrix_diagonal(internal.matrix, value=1.0 * interaction.matrix.diagonal()),
                wrapping_direction=None,
            )
        )


class LineVelocityGaugeOperators(LineLengthGaugeOperators):
    """mesh_operators.py:352-427: the interaction is A(t) times the
    antisymmetric nearest-neighbour coupling i hbar (q/m) / (2 dz); its split
    operators are pair rotations.  ``gauge`` keeps the value the reference
    class declares (mesh_operators.py:355)."""

    gauge = core.Gauge.LENGTH

    def velocity_coefficient(self, mesh):
        """hbar (q/m) / (2 dz): the split angle is tau A times it."""
        spec = mesh.spec
        return float(u.hbar * (spec.test_charge / spec.test_mass) / (2 * mesh.delta_z))

    @_memo
    def interaction_hamiltonian_matrices_without_field(self, mesh):
        off = 1j * self.velocity_coefficient(mesh) * np.ones(len(mesh.z_mesh) - 1, dtype=np.complex128)
        return (sparse.diags((-off, off), offsets=(-1, 1)),)

    def interaction_hamiltonian(self, mesh):
        (m,) = self.interaction_hamiltonian_matrices_without_field(mesh)
        A = mesh.spec.electric_potential.get_vector_potential_amplitude_numeric(mesh.sim.times_to_current)
        return SumOfOperators(DotOperator(A * m, wrapping_direction=None))


# --------------------------------------------------------------------------
# spherical-harmonic mesh
# --------------------------------------------------------------------------


class SphericalHarmonicLengthGaugeOperators(MeshOperators):
    """mesh_operators.py:815-1080.  Both kinetic-energy derivations have a
    device path: the Lagrangian one (the reference default) in every
    precision, the Hamiltonian one in complex128 with the split operator."""

    gauge = core.Gauge.LENGTH

    def __init__(
        self,
        kinetic_energy_derivation=KineticEnergyDerivation.LAGRANGIAN,
        hydrogen_zero_angular_momentum_correction: bool = True,
    ):
        self.kinetic_energy_derivation = KineticEnergyDerivation(kinetic_energy_derivation)
        self.hydrogen_zero_angular_momentum_correction = hydrogen_zero_angular_momentum_correction

    @staticmethod
    def alpha(j):
        x = (j ** 2) + (2 * j)
        return (x + 1) / (x + 0.75)

    @staticmethod
    def beta(j):
        x = 2 * (j ** 2) + (2 * j)
        return (x + 1) / (x + 0.5)

    @staticmethod
    def c_l(l):
        return (l + 1) / np.sqrt(((2 * l) + 1) * ((2 * l) + 3))

    @_memo
    def device_tables(self, mesh):
        """Radial Hamiltonian (kinetic_energy_from_lagrangian + internal
        potential, mesh_operators.py:889-928 and 244-269) and the l-coupling
        factors (interaction_hamiltonian_matrices_without_field, :988-1005).

        Returns a dict with hd [L*Nr] (C order), hoff [Nr-1], rq [Nr], cl [L]
        and the FP64 pieces of the diagonal used by the complex64 path:
        kinv [Nr] (= beta(j) (-2p) + V(r_j)), cent [Nr] and corr0; ``cross``
        is None (the lines are independent).  With
        kinetic_energy_derivation "hamiltonian" the radial Hamiltonian is
        kinetic_energy_from_hamiltonian's (mesh_operators.py:863-887): -2p on
        the diagonal, p between every pair of consecutive points of the
        flattened (l, r) mesh, so also between the last r of each l and the
        first r of the next (``cross`` = p); no l = 0 correction."""
        if self.kinetic_energy_derivation == KineticEnergyDerivation.HAMILTONIAN:
            return self._device_tables_hamiltonian(mesh)
        spec = mesh.spec
        nr, L = spec.r_points, spec.l_bound
        mu = u.electron_mass_reduced
        p = -(u.hbar ** 2) / (2 * mu * (mesh.delta_r ** 2))
        # The reference forms these over the whole flattened mesh, element by
        # element; beta, alpha and V depend on r alone and the centrifugal
        # term on (l, r), so each is formed once per r (or per (l, r)) with
        # the same per-element operations in the same order and broadcast:
        # diag = ((beta_j (+ corr at the first point)) (-2p) + eff) + V.
        beta_r = self.beta(np.arange(nr)).astype(np.float64)
        corr = 0.0
        if self.hydrogen_zero_angular_momentum_correction:
            dr = mesh.delta_r / u.bohr_radius
            corr = dr * (1 + dr) / 8
        V_r = np.asarray(spec.internal_potential(r=mesh.r, test_charge=spec.test_charge), dtype=np.float64)
        r = mesh.r

        def full_hd():  # the (l, r) diagonal: read by the complex128 forms only
            lv = np.arange(L)[:, None]
            eff = ((u.hbar ** 2) / (2 * mu)) * lv * (lv + 1) / (r[None, :] ** 2)
            hd2 = (beta_r * (-2 * p))[None, :] + eff
            hd2[0, 0] = (beta_r[0] + corr) * (-2 * p) + eff[0, 0]
            return (hd2 + V_r[None, :]).reshape(-1)

        hd = core.LazyArray(full_hd)
        hoff = (self.alpha(np.arange(nr - 1)) * p).astype(np.float64)
        rq = -spec.test_charge * mesh.r
        cl = self.c_l(np.arange(L))
        kinv = beta_r * (-2 * p) + V_r
        cent = ((u.hbar ** 2) / (2 * mu)) / (mesh.r ** 2)
        corr0 = (beta_r[0] + corr) * (-2 * p) - beta_r[0] * (-2 * p)
        return dict(hd=hd, hoff=hoff, rq=np.asarray(rq, dtype=np.float64), cl=cl, kinv=kinv, cent=cent,
                    corr0=float(corr0), cross=None)

    def _device_tables_hamiltonian(self, mesh):
        spec = mesh.spec
        nr, L = spec.r_points, spec.l_bound
        mu = u.electron_mass_reduced
        p = -(u.hbar ** 2) / (2 * mu * (mesh.delta_r ** 2))
        diag = p * (-2) * np.ones(nr * L, dtype=np.complex128)
        eff = ((u.hbar ** 2) / (2 * mu)) * mesh.l_mesh * (mesh.l_mesh + 1) / (mesh.r_mesh ** 2)
        diag += eff.flatten("C")
        V = spec.internal_potential(r=mesh.r_mesh, test_charge=spec.test_charge)
        hd = (diag + 1.0 * np.asarray(V).flatten("C")).real.copy()
        V_r = np.asarray(spec.internal_potential(r=mesh.r, test_charge=spec.test_charge), dtype=np.float64)
        return dict(hd=hd, hoff=np.full(nr - 1, p), rq=np.asarray(-spec.test_charge * mesh.r, dtype=np.float64),
                    cl=self.c_l(np.arange(L)), kinv=-2 * p + V_r, cent=((u.hbar ** 2) / (2 * mu)) / (mesh.r ** 2),
                    corr0=0.0, cross=float(p))

    def single_l_hamiltonian(self, mesh, l):
        """(diagonal, off-diagonal) of internal_hamiltonian_for_single_l
        (mesh_operators.py:942-986): the Lagrangian radial kinetic energy of
        one l, its centrifugal term, and V(r), in the reference's order.  The
        reference has no single-l form of the Hamiltonian-derived kinetic
        energy (kinetic_energy_for_single_l_from_hamiltonian raises
        NotImplementedError, :937-940), and neither does this."""
        if self.kinetic_energy_derivation == KineticEnergyDerivation.HAMILTONIAN:
            raise NotImplementedError
        spec = mesh.spec
        nr = spec.r_points
        mu = u.electron_mass_reduced
        p = -(u.hbar ** 2) / (2 * mu * (mesh.delta_r ** 2))
        eff = ((u.hbar ** 2) / (2 * mu)) * l * (l + 1) / (mesh.r ** 2)
        beta = self.beta(np.arange(nr, dtype=np.complex128))
        if l == 0 and self.hydrogen_zero_angular_momentum_correction:
            dr = mesh.delta_r / u.bohr_radius
            beta[0] += dr * (1 + dr) / 8
        diag = (-2 * p * beta) + eff
        off = p * self.alpha(np.arange(nr - 1, dtype=np.complex128))
        V = np.asarray(spec.internal_potential(r=mesh.r, test_charge=spec.test_charge))
        return (diag + V).real.astype(np.float64), off.real.astype(np.float64)

    @_memo
    def internal_hamiltonian(self, mesh):
        t = self.device_tables(mesh)
        nr, L = mesh.spec.r_points, mesh.spec.l_bound
        off = np.zeros(nr * L - 1)
        for l in range(L):
            off[l * nr: l * nr + nr - 1] = t["hoff"]
        if t["cross"] is not None:
            off[nr - 1::nr] = t["cross"]
        m = sparse.diags((off.astype(np.complex128), np.asarray(t["hd"]).astype(np.complex128), off.astype(np.complex128)),
                         offsets=(-1, 0, 1))
        return SumOfOperators(DotOperator(m, wrapping_direction="r"))

    def interaction_hamiltonian(self, mesh):
        t = self.device_tables(mesh)
        L = mesh.spec.l_bound
        efield = mesh.spec.electric_potential.get_electric_field_amplitude(mesh.sim.time + (mesh.spec.time_step / 2))
        rF = mesh.r_mesh.flatten("F")[:-1]
        kk = np.arange(len(rF))
        off = np.where((kk + 1) % L != 0, self.c_l(kk % L), 0) * (-mesh.spec.test_charge * rF)
        m = sparse.diags((off * efield, np.zeros(len(rF) + 1), off * efield), offsets=(-1, 0, 1))
        return SumOfOperators(DotOperator(m, wrapping_direction="l"))


class SphericalHarmonicVelocityGaugeOperators(SphericalHarmonicLengthGaugeOperators):
    """mesh_operators.py:1130-1408: the radial Hamiltonian of the length-gauge
    class; the interaction is h1 + h2 times the vector potential A(t) =
    -integral of E over the times so far (pulses.py:58-77):
      h1 = i hbar (q/m) c_l (l+1) / r between F-order l-neighbours at one r,
      h2 = i hbar (q/m) / (2 dr) kron(c_block, alpha_block)."""

    gauge = core.Gauge.VELOCITY

    def __init__(self, hydrogen_zero_angular_momentum_correction: bool = True):
        super().__init__(hydrogen_zero_angular_momentum_correction=hydrogen_zero_angular_momentum_correction)

    def __repr__(self):
        return (f"{self.__class__.__name__}(hydrogen_zero_angular_momentum_correction = "
                f"{self.hydrogen_zero_angular_momentum_correction})")

    @_memo
    def velocity_tables(self, mesh):
        """rq [Nr] = hbar (q/m) / r_j (h1 = A rq_j c_l (l+1) between l-neighbours)
        and h2r [Nr-1] = hbar (q/m) / (2 dr) alpha(j) (h2 = A c_l h2r_j on the
        (l, j)-(l+1, j+1) link)."""
        spec = mesh.spec
        q_over_m = spec.test_charge / spec.test_mass
        rq = (u.hbar * q_over_m) / mesh.r
        h2r = (u.hbar * q_over_m / (2 * mesh.delta_r)) * self.alpha(np.arange(spec.r_points - 1))
        return dict(rq=np.asarray(rq, dtype=np.float64), h2r=np.asarray(h2r, dtype=np.float64))

    @_memo
    def interaction_hamiltonian_matrices_without_field(self, mesh):
        """(h1, h2) as sparse matrices (mesh_operators.py:1143-1176); h1 acts on
        the mesh flattened along l, h2 along r."""
        spec = mesh.spec
        L, nr = spec.l_bound, spec.r_points
        q_over_m = spec.test_charge / spec.test_mass
        rF = mesh.r_mesh.flatten("F")[:-1]
        kk = np.arange(len(rF))
        l_of = kk % L
        h1_off = np.where((kk + 1) % L != 0, self.c_l(l_of) * (l_of + 1), 0) * (1j * u.hbar * q_over_m) / rF
        h1 = sparse.diags((-h1_off, h1_off), offsets=(-1, 1))
        alpha_vec = self.alpha(np.arange(nr - 1, dtype=np.complex128))
        c_vec = self.c_l(np.arange(L - 1, dtype=np.complex128))
        h2 = (1j * u.hbar * q_over_m / (2 * mesh.delta_r)) * sparse.kron(
            sparse.diags((c_vec, c_vec), offsets=(-1, 1)), sparse.diags((-alpha_vec, alpha_vec), offsets=(-1, 1)),
            format="dia")
        return h1, h2

    def interaction_hamiltonian(self, mesh):
        h1, h2 = self.interaction_hamiltonian_matrices_without_field(mesh)
        A = mesh.spec.electric_potential.get_vector_potential_amplitude_numeric(mesh.sim.times_to_current)
        return SumOfOperators(DotOperator(A * h1, wrapping_direction="l"), DotOperator(A * h2, wrapping_direction="r"))


# --------------------------------------------------------------------------
# cylindrical slice mesh
# --------------------------------------------------------------------------


class RectangleLengthGaugeOperators(MeshOperators):
    """mesh_operators.py:430-505: kinetic energies along z then x (uniform
    second differences), half of the internal potential and half of
    -z q E(t) on each diagonal (mesh_operators.py:244-298)."""

    gauge = core.Gauge.LENGTH

    @_memo
    def device_tables(self, mesh):
        """Diagonals of the internal H_z and H_x in C order of the (z, x) mesh,
        their (uniform) off-diagonals, and zq = -z * test_charge."""
        spec = mesh.spec
        nz, nx = spec.z_points, spec.x_points
        m = spec.test_mass
        pz = -(u.hbar ** 2) / (2 * m * (mesh.delta_z ** 2))
        px = -(u.hbar ** 2) / (2 * m * (mesh.delta_x ** 2))
        V = np.asarray(spec.internal_potential(r=mesh.r_mesh, z=mesh.z_mesh, x=mesh.x_mesh, test_charge=spec.test_charge),
                       dtype=np.float64) * np.ones((nz, nx))
        hz_d = (pz * (-2) + 0.5 * V).reshape(-1)
        hr_d = (px * (-2) + 0.5 * V).reshape(-1)
        zq = -mesh.z * spec.test_charge
        return dict(hz_d=hz_d, hz_off=pz * np.ones(nz - 1), hr_d=hr_d, hr_off=px * np.ones(nx - 1),
                    zq=np.asarray(zq, dtype=np.float64))


class SphericalSliceLengthGaugeOperators(MeshOperators):
    """mesh_operators.py:693-813: kinetic energies along theta (a
    non-symmetric tridiagonal) then r, half of the internal potential and
    half of -z q E(t) on each diagonal.  ``gauge`` keeps the value the
    reference class declares (mesh_operators.py:696)."""

    gauge = core.Gauge.VELOCITY

    @_memo
    def device_tables(self, mesh):
        """The theta operator T = P_theta / (j + 1/2)^2 x [upper, -2, lower]
        (mesh_operators.py:724-775) is D S D^-1 with S symmetric and D =
        diag(d_k) in theta alone: d_{k+1}/d_k = sqrt(lower_k / upper_k) does
        not depend on j, so D commutes with the r operator and with every
        diagonal term, and the step runs on psi' = D^-1 g with S.  Returns
        the r (strided) and theta (contiguous) tables of the two-direction ADI
        kernels, the per-row theta factor 1/(j + 1/2)^2, z q per point, and D."""
        spec = mesh.spec
        nr, nth = spec.r_points, spec.theta_points
        mu = u.electron_mass_reduced
        dr, dth = mesh.delta_r, mesh.delta_theta
        pt = -(u.hbar ** 2) / (2 * mu * ((dr * dth) ** 2))
        pr = -(u.hbar ** 2) / (2 * mu * (dr ** 2))
        j = np.arange(nr)
        tjp = 1 / (j + 0.5) ** 2
        k = np.arange(nth - 1)
        c = lambda x: (dth / 2) / np.tan(x * dth)  # noqa: E731
        sk = lambda x: np.sin(x * dth)  # noqa: E731
        up = (1 + c(k + 0.5)) * np.sqrt(sk(k + 0.5) / sk(k + 1.5))
        lo = (1 - c(k + 1.5)) * np.sqrt(sk(k + 1.5) / sk(k + 0.5))
        d = np.concatenate([[1.0], np.cumprod(np.sqrt(lo / up))])
        V = np.asarray(spec.internal_potential(r=mesh.r_mesh, test_charge=spec.test_charge), dtype=np.float64)
        V = V * np.ones((nr, nth))
        hr_d = ((-2 * pt) * tjp[:, None] + 0.5 * V).reshape(-1)  # theta diagonal, C order
        hz_d = ((-2 * pr) + 0.5 * V).reshape(-1)  # r diagonal
        zq_pt = (-spec.test_charge * mesh.r_mesh * np.cos(mesh.theta_mesh)).reshape(-1)
        return dict(hz_d=hz_d, hz_off=pr * np.ones(nr - 1), hr_d=hr_d, hr_off=pt * np.sqrt(up * lo),
                    hr_off_row=tjp, zq_pt=zq_pt, d=d)


class CylindricalSliceLengthGaugeOperators(MeshOperators):
    """mesh_operators.py:550-640."""

    gauge = core.Gauge.LENGTH

    @_memo
    def device_tables(self, mesh):
        """Diagonals of the internal H_z and H_rho (each with half of V,
        mesh_operators.py:244-269) in C order of the (z, rho) mesh, their
        off-diagonals, and zq = -z * test_charge."""
        spec = mesh.spec
        nz, nr = spec.z_points, spec.rho_points
        M = nz * nr
        m = spec.test_mass
        pz = -(u.hbar ** 2) / (2 * m * (mesh.delta_z ** 2))
        prho = -(u.hbar ** 2) / (2 * m * (mesh.delta_rho ** 2))
        z_diag = pz * (-2) * np.ones(M, dtype=np.complex128)
        rho_diag = prho * (-2) * np.ones(M, dtype=np.complex128)
        jj = np.arange(1, nr)
        cj = jj / np.sqrt((jj ** 2) - 0.25)
        hr_off = (cj.astype(np.complex128) * prho).real.copy()
        hz_off = (pz * np.ones(nz - 1, dtype=np.complex128)).real.copy()
        V = spec.internal_potential(r=mesh.r_mesh, z=mesh.z_mesh, test_charge=spec.test_charge)
        pre = 1 / 2
        hz_d_F = (z_diag + pre * np.asarray(V).flatten("F")).real
        hz_d = np.reshape(hz_d_F, (nz, nr), "F").flatten("C")
        hr_d = (rho_diag + pre * np.asarray(V).flatten("C")).real.copy()
        zq = -mesh.z * spec.test_charge
        return dict(hz_d=hz_d, hz_off=hz_off, hr_d=hr_d, hr_off=hr_off, zq=np.asarray(zq, dtype=np.float64))
