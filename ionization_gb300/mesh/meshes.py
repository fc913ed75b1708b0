"""Meshes: grids, the device-resident wavefunction ``g`` and data reductions.

Grids, state projection and inner-product conventions follow
ionization/mesh/meshes.py (LineMesh :263-341, CylindricalSliceMesh :509-607,
SphericalHarmonicMesh :985-1136).  The wavefunction lives on the GPU between
steps; ``mesh.g`` is a host copy made on access (and uploaded on assignment),
so datastores and user code see the reference's array shapes:
line (z_points,), spherical harmonic (l_bound, r_points), cylindrical
(z_points, rho_points).
"""

import ctypes
from typing import Optional

import numpy as np
import torch

from .. import _device as dev
from .. import _native as nat
from .. import core, exceptions, potentials, states
from .. import units as u
from . import evolution_methods as em
from . import mesh_operators as mo


class WrappingDirection(core.StrEnum):
    X = "x"
    Y = "y"
    Z = "z"
    RHO = "rho"
    CHI = "chi"
    THETA = "theta"
    R = "r"
    L = "l"


class QuantumMesh:
    """Base mesh.  Subclasses set the grid, ``mesh_shape``, ``inner_product_multiplier``,
    ``g_factor`` and build their device state in ``_init_device``."""

    fused_data = True  # data reductions happen inside the step kernels

    def __init__(self, sim):
        self.sim = sim
        self.spec = sim.spec
        self.operators = self.spec.operators
        self.precision = core.Precision(getattr(self.spec, "precision", core.Precision.C128))
        self.inner_product_multiplier = None

    # ---- layout helpers (meshes.py:117-133) ----
    def wrapping_direction_to_order(self, wrapping_direction) -> Optional[str]:
        return None

    def flatten_mesh(self, mesh, flatten_along):
        order = self.wrapping_direction_to_order(flatten_along)
        return mesh if order is None else mesh.flatten(order)

    def wrap_vector(self, vector, wrap_along):
        order = self.wrapping_direction_to_order(wrap_along)
        return vector if order is None else np.reshape(vector, self.mesh_shape, order)

    # ---- wavefunction ----
    def _psi_residual(self):
        """The device residual of psi (precision c64x), else None."""
        return None

    @property
    def g(self) -> np.ndarray:
        g = self._psi_device().cpu().numpy().astype(np.complex128)
        lo = self._psi_residual()
        if lo is not None:
            g = g + dev.lo_unpack(lo.cpu().numpy()).reshape(g.shape)
        return g.reshape(self.mesh_shape)

    @g.setter
    def g(self, value):
        d = self._psi_device()
        v = np.ascontiguousarray(np.asarray(value, dtype=np.complex128).reshape(d.shape))
        d.copy_(torch.from_numpy(v).to(d.device, d.dtype))
        lo = self._psi_residual()
        if lo is not None:
            hi = v.astype(np.complex64).astype(np.complex128)
            lo.copy_(torch.from_numpy(dev.lo_pack(v - hi)).to(lo.device))

    def _native_state(self):
        """Host copies of the device arrays that hold psi (the state itself and,
        in the c64x form, its residual), for an exact save and restore."""
        lo = self._psi_residual()
        return (self._psi_device().cpu().numpy().copy(), None if lo is None else lo.cpu().numpy().copy())

    def _set_native_state(self, state):
        hi, lo = state
        self._psi_device().copy_(torch.from_numpy(np.ascontiguousarray(hi)).to(self._psi_device().device))
        if lo is not None and self._psi_residual() is not None:
            self._psi_residual().copy_(torch.from_numpy(np.ascontiguousarray(lo)).to(self._psi_residual().device))

    @property
    def psi(self):
        return self.g / self.g_factor

    @property
    def g2(self):
        return np.abs(self.g) ** 2

    @property
    def psi2(self):
        return np.abs(self.psi) ** 2

    # ---- states and inner products (meshes.py:135-217) ----
    def state_to_g(self, state_or_mesh):
        if state_or_mesh is None:
            return self.g
        if isinstance(state_or_mesh, states.QuantumState):
            return self.get_g_for_state(state_or_mesh)
        return state_or_mesh

    def inner_product(self, a=None, b=None):
        return np.sum(np.conj(self.state_to_g(a)) * self.state_to_g(b)) * self.inner_product_multiplier

    def state_overlap(self, a=None, b=None):
        return np.abs(self.inner_product(a, b)) ** 2

    def norm(self, state=None):
        return self.inner_product(state, state).real

    # ---- position expectation values and partial norms (device reductions) ----
    def _weighted_norms(self, weights):
        """weight * sum w |g|^2 for each weight array (mesh shape), on the device."""
        import torch

        out = []
        g = self._psi_device()
        lo = self._psi_residual()
        n = int(np.prod(self.mesh_shape))
        for k0 in range(0, len(weights), 8):
            chunk = weights[k0:k0 + 8]
            w = np.stack([np.broadcast_to(np.asarray(x, dtype=np.float64), self.mesh_shape).reshape(-1)
                          for x in chunk])
            d_w = dev.to_dev(w)
            nbytes = nat.value("ion_weighted_norms_scratch_bytes", n, len(chunk))
            scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=g.device)
            res = torch.empty(len(chunk), dtype=torch.float64, device=g.device)
            if g.dtype == torch.complex128:
                nat.call("ion_weighted_norms_c128", n, dev.ptr(g), len(chunk), dev.ptr(d_w),
                         float(self.inner_product_multiplier), dev.ptr(res), dev.ptr(scratch), int(nbytes),
                         dev.stream_ptr())
            else:
                nat.call("ion_weighted_norms_c64", n, dev.ptr(g), dev.ptr(lo), len(chunk), dev.ptr(d_w),
                         float(self.inner_product_multiplier), dev.ptr(res), dev.ptr(scratch), int(nbytes),
                         dev.stream_ptr())
            out.extend(res.cpu().numpy().tolist())
        return out

    def z_expectation_value(self):
        """<z> of the current wavefunction (meshes.py:231-233)."""
        return self._weighted_norms([self.z_mesh])[0]

    def r_expectation_value(self):
        """<r> of the current wavefunction (meshes.py:235-237)."""
        return self._weighted_norms([self.r_mesh])[0]

    def norm_within_radius(self, radii):
        """The norm of the mesh points with r <= R, for each R (data.py:420-425)."""
        return self._weighted_norms([(self.r_mesh <= R).astype(np.float64) for R in radii])

    # ---- energy expectation values (device reductions) ----
    def _energy_operators(self):
        """((n_a, n_b), internal, interaction, field): the internal
        Hamiltonian and the interaction per unit field as (diag, off_b, off_a,
        flags) tables over the (n_a, n_b) C-order layout of g (each array
        broadcast to the mesh, off-diagonals indexed by the point they start
        from; ion_hop), and ``field()`` the interaction's field factor at the
        current time.  interaction None: the total Hamiltonian has no
        interaction term; the string "unsupported": the device has no form of
        it."""
        raise exceptions.UnsupportedMesh(f"no energy expectation values on {type(self).__name__}")

    def _energy_device(self):
        if getattr(self, "_d_energy", None) is None:
            (na, nb), internal, inter, field = self._energy_operators()
            ops = [internal] + ([inter] if isinstance(inter, tuple) else [])
            hops = (nat.Hop * len(ops))()
            keep = []
            for q, (diag, off_b, off_a, flags) in enumerate(ops):
                for name, arr in (("diag", diag), ("off_b", off_b), ("off_a", off_a)):
                    if arr is not None:
                        full = np.broadcast_to(np.asarray(arr, dtype=np.float64), (na, nb)).reshape(-1)
                        keep.append(dev.to_dev(full))
                        setattr(hops[q], name, dev.ptr(keep[-1]))
                hops[q].flags = int(flags)
            self._d_energy = (na, nb, hops, keep, inter, field)
        return self._d_energy

    def _energy_terms(self):
        """weight * <g|H0|g> and, when the mesh has one, weight * <g|V|g> with
        V the interaction per unit field, in one device pass."""
        import torch

        na, nb, hops, _, inter, field = self._energy_device()
        g = self._psi_device()
        lo = self._psi_residual()
        nbytes = nat.value("ion_expectation_scratch_bytes", na, nb, len(hops))
        scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=g.device)
        res = torch.empty(len(hops), dtype=torch.float64, device=g.device)
        ops = ctypes.cast(hops, ctypes.c_void_p)
        w = float(self.inner_product_multiplier)
        if g.dtype == torch.complex128:
            nat.call("ion_expectation_c128", dev.ptr(g), na, nb, len(hops), ops, w, dev.ptr(res), dev.ptr(scratch),
                     int(nbytes), dev.stream_ptr())
        else:
            nat.call("ion_expectation_c64", dev.ptr(g), dev.ptr(lo), na, nb, len(hops), ops, w, dev.ptr(res),
                     dev.ptr(scratch), int(nbytes), dev.stream_ptr())
        return res.cpu().numpy(), inter, field

    def internal_energy_expectation_value(self):
        """<H0> of the current wavefunction: the internal Hamiltonian
        (kinetic energy and internal potential, mesh_operators.py:244-269;
        QuantumMesh.internal_energy_expectation_value, meshes.py:219-223)."""
        return float(self._energy_terms()[0][0])

    def total_energy_expectation_value(self):
        """<H0 + V(t)> of the current wavefunction: the internal Hamiltonian
        plus the interaction at the current time (total_hamiltonian,
        mesh_operators.py:271-298; meshes.py:225-229)."""
        if self._energy_device()[4] == "unsupported":
            raise exceptions.UnsupportedMesh(
                f"{type(self.operators).__name__} on {type(self).__name__}: no device form of the interaction energy")
        v, inter, field = self._energy_terms()
        return float(v[0]) if inter is None else float(v[0] + field() * v[1])

    # ---- stepping ----
    def _method_supported(self):
        raise NotImplementedError

    def _device_evolve(self, method, time_step):
        """One step through the device path; ``time_step`` replaces the
        tabulated step of the current time index if it differs."""
        t = self.sim.time_index
        tau = time_step / (2 * u.hbar)
        self._set_tau(t, tau)
        self._evolve_steps(1)
        return self._psi_device()

    def evolve(self, time_step):
        """QuantumMesh.evolve (meshes.py:251-257): one step then the mask."""
        self.spec.evolution_method.evolve(self, None, time_step)

    def _set_tau(self, t_now, tau):
        if self._tau_host[t_now] != tau:
            self._tau_host[t_now] = tau
            self._tau_dev()[t_now] = tau


def sph_harm_m0(ls, theta) -> np.ndarray:
    """Y_l^0(theta) = sqrt((2l + 1) / 4 pi) P_l(cos theta) for each l of
    ``ls`` (rows) at each theta (columns), P_l by the three-term recurrence
    (n + 1) P_{n+1} = (2n + 1) x P_n - n P_{n-1}: the values scipy's
    sph_harm(0, l, 0, theta) gives the reference (meshes.py:1487-1490)."""
    ls = np.asarray(ls, dtype=int)
    x = np.cos(np.asarray(theta, dtype=np.float64))
    lmax = int(ls.max()) if ls.size else 0
    p = np.empty((lmax + 1, x.size))
    p[0] = 1.0
    if lmax >= 1:
        p[1] = x
    for n in range(1, lmax):
        p[n + 1] = ((2 * n + 1) * x * p[n] - n * p[n - 1]) / (n + 1)
    return np.sqrt((2 * ls[:, None] + 1) / (4 * np.pi)) * p[ls]


def _two_axis_energy_operators(mesh, n_a, n_b):
    """Energy operators of a (z, b) mesh whose internal Hamiltonian is
    H_z + H_b (each kinetic operator with its share of the potential,
    mesh_operators.py:244-269, device_tables): diagonal hz_d + hr_d,
    couplings hz_off along z and hr_off along b; the interaction per unit
    field is -q z on the diagonal times E(t) (interaction_hamiltonian,
    mesh_operators.py:475-497, 605-627: split over the two directions and
    summed back by total_hamiltonian, :271-298)."""
    tb = mesh.operators.device_tables(mesh)
    diag = (np.asarray(tb["hz_d"], dtype=np.float64) + np.asarray(tb["hr_d"], dtype=np.float64)).reshape(n_a, n_b)
    off_b = np.append(np.asarray(tb["hr_off"], dtype=np.float64), 0.0)
    off_a = np.append(np.asarray(tb["hz_off"], dtype=np.float64), 0.0)[:, None]
    internal = (diag, off_b, off_a, 0)
    inter = (np.asarray(tb["zq"], dtype=np.float64)[:, None], None, None, 0)
    spec, sim = mesh.spec, mesh.sim
    return (n_a, n_b), internal, inter, lambda: float(spec.electric_potential.get_electric_field_amplitude(sim.time))


def _radial_states_array(gs, n_r) -> np.ndarray:
    """The test states' radial g as one [n_states, n_r] array: float64 when
    every value is real (hydrogen and numeric eigenstates), so the device
    reads (and the upload moves) one double a point, else complex128."""
    a = np.array(gs, dtype=np.complex128).reshape(len(gs), n_r)
    return a.real.copy() if a.size and not np.any(a.imag) else a


def _adi_precision(mesh, what):
    """The two-direction ADI kernel pair has complex128 and complex64 forms
    (FP32 sweeps, FP64 tables and reductions); the stored-residual form
    (c64x) is the spherical-harmonic split and line kernels' only."""
    if mesh.precision == core.Precision.C64X:
        raise exceptions.UnsupportedMesh(
            f"the {what} device path has complex128 and complex64 forms, no c64x (stored residual) form")


def _adi_cap(mesh):
    """Longest line of the ADI kernel pair at the mesh's precision."""
    if getattr(mesh.spec, "host_only", False):
        return 1 << 62
    return nat.value("ion_cyl_max_points_" + ("c128" if mesh.precision == core.Precision.C128 else "c64"))


class _AdiDevice:
    """Device state of a mesh advanced by the two-direction ADI kernel pair
    (``ion_cyl_adi_run_c128`` / ``_c64``: a pass implicit along the strided direction,
    then one implicit along the contiguous one), with whole-mesh reductions
    at data times.  Used by the cylindrical slice mesh (z, rho) and by the
    spherical-harmonic mesh under AlternatingDirectionImplicit (l, r)."""

    fused_data = False

    def _adi_setup(self, n_strided, n_contig, arrays, g0, test_g):
        """``arrays``: the ion_cyl_mesh tables by field name (FP64, or None)."""
        f64 = np.float64
        self._d = {k: (dev.to_dev(np.asarray(v).reshape(-1), f64) if v is not None else None) for k, v in arrays.items()}
        cdt = np.complex128 if self.precision == core.Precision.C128 else np.complex64
        self._g = dev.to_dev(np.asarray(g0, dtype=np.complex128).astype(cdt))
        self._gtmp = torch.empty_like(self._g)
        cm = nat.CylMesh()
        cm.n_z, cm.n_rho = int(n_strided), int(n_contig)
        for k, v in self._d.items():
            setattr(cm, k, dev.ptr(v))
        self._cm = cm
        self._reducer = dev.Reducer(self.mesh_points, test_g, self.inner_product_multiplier)
        self._t = 0
        times = self.sim.times
        self.n_data = dev.n_data_slots(len(times) - 1, self.spec.store_data_every)
        self._d_norm = torch.full((self.n_data,), float("nan"), dtype=torch.float64, device=dev.device())
        self._d_ip = torch.full((self.n_data, max(len(test_g), 1), 2), float("nan"), dtype=torch.float64,
                                device=dev.device())

    def _adi_evolve_steps(self, n):
        fn = "ion_cyl_adi_run_c128" if self._g.dtype == torch.complex128 else "ion_cyl_adi_run_c64"
        nat.call(fn, self._cm, dev.ptr(self._g), dev.ptr(self._gtmp), self._t, int(n), dev.stream_ptr())
        self._t += int(n)

    def _adi_reduce_current(self):
        tf = len(self.sim.times) - 1
        slot = dev.data_slot(self._t, tf, self.spec.store_data_every)
        self._reducer(self._g, self._d_norm[slot:slot + 1], self._d_ip[slot])

    def _adi_pull_data(self):
        norm = self._d_norm.cpu().numpy()
        ns = len(self.spec.test_states)
        ip = self._d_ip.cpu().numpy()[:, :ns, :].copy().view(np.complex128)[..., 0]
        return norm, ip.T.copy()


# ==========================================================================
# line
# ==========================================================================


class LineMesh(QuantumMesh):
    mesh_storage_method = ("z",)

    def __init__(self, sim):
        super().__init__(sim)
        self.z_mesh = np.linspace(-self.spec.z_bound, self.spec.z_bound, self.spec.z_points)
        self.delta_z = np.abs(self.z_mesh[1] - self.z_mesh[0])
        self.z_center_index = int(np.argmin(np.abs(self.z_mesh)))
        self.mesh_points = len(self.z_mesh)
        self.mesh_shape = (self.mesh_points,)
        self.inner_product_multiplier = self.delta_z
        self.g_factor = 1
        self._state_g_cache = {}
        self._init_device()

    @property
    def z(self):
        return self.z_mesh

    @property
    def r(self):
        return self.z

    @property
    def r_mesh(self):
        return self.z_mesh

    def get_g_for_state(self, state):
        """LineMesh.get_g_for_state (meshes.py:327-341)."""
        if state in self._state_g_cache:
            return self._state_g_cache[state]
        g = state(self.z_mesh)
        g = g / np.sqrt(np.sum(np.conj(g) * g).real * self.inner_product_multiplier)
        g = g * state.amplitude
        self._state_g_cache[state] = g
        return g

    def _init_device(self):
        spec, sim = self.spec, self.sim
        method = spec.evolution_method
        if not isinstance(self.operators, mo.LineLengthGaugeOperators):
            raise exceptions.UnsupportedMesh(f"{type(self.operators).__name__} has no device path on LineMesh")

        if isinstance(method, em.AlternatingDirectionImplicit):
            kind = nat.ION_LINE_ADI
        elif isinstance(method, em.SplitInteractionOperator):
            kind = nat.ION_LINE_SPLIT
        elif isinstance(method, em.FourierSplitOperator):
            kind = nat.ION_LINE_FFT
        else:
            raise exceptions.UnsupportedMesh(f"{type(method).__name__} has no device path on LineMesh")
        hd, hoff, zq = self.operators.device_tables(self)
        vstat = kin = twiddle = None
        if kind == nat.ION_LINE_FFT and self.precision == core.Precision.C64X:
            raise exceptions.UnsupportedMesh("FourierSplitOperator has no c64x (stored residual) form")
        if kind == nat.ION_LINE_FFT:
            try:
                vstat, kin, twiddle = self.operators.fourier_tables(self)
            except ValueError as e:
                raise exceptions.UnsupportedMesh(str(e)) from e
        mask = spec.mask(r=self.r_mesh)
        mask = None if np.isscalar(mask) and mask == 1 else np.broadcast_to(np.asarray(mask, np.float64), (self.mesh_points,))
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        efield = np.zeros(len(times))
        gauge, vcoef = nat.ION_GAUGE_LENGTH, 0.0
        if isinstance(self.operators, mo.LineVelocityGaugeOperators):
            if kind != nat.ION_LINE_SPLIT:
                raise exceptions.UnsupportedMesh("LineVelocityGaugeOperators have a device path with SplitInteractionOperator only")
            if self.precision == core.Precision.C64X:
                raise exceptions.UnsupportedMesh("LineVelocityGaugeOperators have no c64x (stored residual) form")
            gauge, vcoef = nat.ION_GAUGE_VELOCITY, self.operators.velocity_coefficient(self)
            efield[1:] = potentials.vector_potential_table(spec.electric_potential, times)[1:]
        else:
            efield[1:] = np.asarray(spec.electric_potential.get_electric_field_amplitude(times[1:]), np.float64) * np.ones(len(times) - 1)
        test_g = np.array([self.get_g_for_state(s) for s in spec.test_states], dtype=np.complex128).reshape(-1, self.mesh_points)
        g0 = self.get_g_for_state(spec.initial_state)
        if not getattr(spec, "host_only", False):
            cta = dev.line_cta_max_n(self.precision)
            maxn = cta if kind == nat.ION_LINE_FFT or gauge == nat.ION_GAUGE_VELOCITY else cta * dev.LINE_MAX_CLUSTER
            if self.mesh_points > maxn:
                raise exceptions.UnsupportedMesh(
                    f"line of {self.mesh_points} points exceeds the device limit {maxn} for {type(method).__name__}")
        self.tables = dev.LineTables(
            n=self.mesh_points, method=kind, hd=hd, hoff=hoff, zq=zq, mask=mask, tau=self._tau_host.copy(),
            efield=efield, state_g=test_g, weight=self.inner_product_multiplier, g0=g0, t0=0,
            t_final=len(times) - 1, store_every=spec.store_data_every, vstat=vstat, kin=kin, twiddle=twiddle,
            gauge=gauge, vcoef=vcoef,
        )
        if getattr(spec, "host_only", False):
            return
        self._dsim = dev.LineDeviceSim(self.tables, self.precision)
        self._batch = dev.LineBatch(self.precision, [self._dsim])

    def _psi_device(self):
        return self._dsim.g

    def _psi_residual(self):
        return self._dsim.g_lo

    def _energy_operators(self):
        """H0 = diag(hd) + hoff couplings along z; the interaction per unit
        field: -q z on the diagonal times E(t) (length gauge,
        mesh_operators.py:320-327).  The velocity gauge's interaction
        (:358-382) has no diagonal, and the line's total_hamiltonian adds only
        the interaction's diagonal to H0 (mesh_operators.py:271-298), so its
        total energy is the internal one."""
        hd, hoff, zq = self.operators.device_tables(self)
        internal = (hd, np.append(hoff, 0.0), None, 0)
        if isinstance(self.operators, mo.LineVelocityGaugeOperators):
            return (1, self.mesh_points), internal, None, None
        spec, sim = self.spec, self.sim
        return (1, self.mesh_points), internal, (zq, None, None, 0), lambda: float(
            spec.electric_potential.get_electric_field_amplitude(sim.time))

    def _tau_dev(self):
        return self._dsim.d_tau

    def _evolve_steps(self, n):
        self._batch.run(n)

    def _reduce_current(self):
        self._batch.reduce()

    def _pull_data(self):
        return self._dsim.data()


# ==========================================================================
# spherical harmonic
# ==========================================================================


class SphericalHarmonicMesh(_AdiDevice, QuantumMesh):
    mesh_storage_method = ("l", "r")
    fused_data = True  # False under AlternatingDirectionImplicit

    def __init__(self, sim):
        super().__init__(sim)
        self.r = np.linspace(0, self.spec.r_bound, self.spec.r_points)
        self.delta_r = self.r[1] - self.r[0]
        self.r = self.r + self.delta_r / 2
        self.r_max = np.max(self.r)
        self.inner_product_multiplier = self.delta_r
        self.l = np.array(range(self.spec.l_bound), dtype=int)
        self.mesh_points = len(self.r) * len(self.l)
        # read-only broadcast views (the grid is never written through them)
        self.l_mesh, self.r_mesh = np.meshgrid(self.l, self.r, indexing="ij", copy=False)
        self.mesh_shape = np.shape(self.r_mesh)
        self._radial_cache = {}
        if self.spec.use_numeric_eigenstates:  # meshes.py:1021-1033
            self.analytic_to_numeric = self.get_numeric_eigenstate_basis(
                self.spec.numeric_eigenstate_max_energy, self.spec.numeric_eigenstate_max_angular_momentum)
            self.spec.test_states = sorted(self.analytic_to_numeric.values(), key=lambda x: x.energy)
            if not self.spec.initial_state.numeric:
                self.spec.initial_state = self.analytic_to_numeric[self.spec.initial_state]
        self._init_device()

    def get_numeric_eigenstate_basis(self, max_energy, max_angular_momentum):
        """meshes.py:1281-1356: for each l <= max_angular_momentum the
        eigenpairs of the single-l Hamiltonian with energy <= max_energy (at
        most r_points - 2, the smallest), normalised on the mesh and divided by
        the g factor, labelled by the analytic state they approximate (bound:
        HydrogenBoundState(n = int(sqrt(rydberg / |E|)), l); free:
        HydrogenCoulombState(E, l)).  The reference takes them from scipy's
        eigsh on each matrix in turn; here all l are solved together on the
        device (batched Sturm bisection and inverse iteration).  Eigenvectors
        are real with a fixed sign; the reference's carry an arbitrary phase."""
        L = int(max_angular_momentum) + 1
        mats = [self.operators.single_l_hamiltonian(self, l) for l in range(L)]
        nr = self.spec.r_points
        pairs = dev.tridiagonal_eigenpairs(np.array([m[0] for m in mats]), np.array([m[1] for m in mats]),
                                           max_energy, nr - 2)
        basis = {}
        for l, (vals, vecs) in enumerate(pairs):
            for energy, v in zip(vals, vecs):
                v = v / np.sqrt(self.inner_product_multiplier * np.sum(np.abs(v) ** 2))
                v = v / self.g_factor
                if energy > max_energy:
                    continue
                if energy > 0:
                    analytic = states.HydrogenCoulombState(energy=energy, l=l)
                    binding = states.Binding.FREE
                else:
                    n_guess = max(1, int(np.sqrt(u.rydberg / np.abs(energy))))
                    analytic = states.HydrogenBoundState(n=n_guess, l=l)
                    binding = states.Binding.BOUND
                basis[analytic] = states.NumericSphericalHarmonicState(
                    g=v, l=l, m=0, energy=energy, corresponding_analytic_state=analytic, binding=binding)
        return basis

    @property
    def g_factor(self):
        return self.r

    def wrapping_direction_to_order(self, wrapping_direction):
        if wrapping_direction is None:
            return None
        if wrapping_direction == WrappingDirection.L:
            return "F"
        if wrapping_direction == WrappingDirection.R:
            return "C"
        raise ValueError(f"{wrapping_direction} is not a valid specifier for flatten_mesh (valid specifiers: 'l', 'r')")

    def get_radial_g_for_state(self, state):
        """meshes.py:1089-1097: R(r) * r normalised on the radial grid."""
        if state in self._radial_cache:
            return self._radial_cache[state]
        g = state.radial_function(self.r) * self.g_factor
        g = g / np.sqrt(np.sum(np.conj(g) * g).real * self.inner_product_multiplier)
        g = g * state.amplitude
        g = np.asarray(g, dtype=np.complex128)
        self._radial_cache[state] = g
        return g

    def get_g_for_state(self, state):
        """meshes.py:1066-1087."""
        rows, vals = self._g_rows_for_state(state)
        g = np.zeros(self.mesh_shape, dtype=np.complex128)
        for l, v in zip(rows, vals):
            g[l, :] = v
        return g

    def _g_rows_for_state(self, state):
        """The l rows of get_g_for_state(state) that hold its components
        (sorted) and their values: each component's radial g added into its
        row in component order, as the full-mesh form adds them."""
        if not all(hasattr(s, "radial_function") for s in state):
            raise NotImplementedError(
                "States with non-definite angular momentum components are not currently supported by SphericalHarmonicMesh"
            )
        if state.analytic and getattr(self.spec, "use_numeric_eigenstates", False):
            state = getattr(self, "analytic_to_numeric", {}).get(state, state)
        acc = {}
        for s in state:
            if not 0 <= s.l < self.spec.l_bound:
                raise IndexError(f"state component with l = {s.l} outside the mesh's l_bound {self.spec.l_bound}")
            if s.l not in acc:
                acc[s.l] = np.zeros(self.spec.r_points, dtype=np.complex128)
            acc[s.l] += self.get_radial_g_for_state(s)
        rows = sorted(acc)
        return rows, [acc[l] for l in rows]

    def inner_product(self, a=None, b=None):
        """The per-l shortcut of meshes.py:1099-1131 when ``a`` is a state and
        ``b`` the current wavefunction."""
        if isinstance(a, states.QuantumState) and all(hasattr(s, "radial_function") for s in a) and b is None:
            g = self.g
            ip = 0
            for s in a:
                ip += np.sum(np.conj(self.get_radial_g_for_state(s)) * g[s.l, :])
            return ip * self.inner_product_multiplier
        return super().inner_product(a, b)

    def norm_by_l(self, state=None):
        g = self.state_to_g(state)
        return np.abs(np.sum(np.conj(g) * g, axis=1) * self.delta_r)

    def _init_device(self):
        spec, sim = self.spec, self.sim
        self._adi = False
        if not isinstance(self.operators, mo.SphericalHarmonicLengthGaugeOperators):
            raise exceptions.UnsupportedMesh(f"{type(self.operators).__name__} has no device path on SphericalHarmonicMesh")
        derivation = getattr(self.operators, "kinetic_energy_derivation", None)
        hamiltonian = derivation == mo.KineticEnergyDerivation.HAMILTONIAN
        if hamiltonian and (self.precision != core.Precision.C128 or
                            not isinstance(spec.evolution_method, em.SplitInteractionOperator)):
            raise exceptions.UnsupportedMesh(
                "kinetic_energy_derivation='hamiltonian' has a device path in complex128 with "
                "SplitInteractionOperator only")
        if isinstance(spec.evolution_method, em.AlternatingDirectionImplicit):
            return self._init_device_adi()
        if not isinstance(spec.evolution_method, em.SplitInteractionOperator):
            raise exceptions.UnsupportedMesh(
                f"{type(spec.evolution_method).__name__} has no device path on SphericalHarmonicMesh"
            )
        suffix = "c128" if self.precision == core.Precision.C128 else "c64"
        maxr = 1 << 62 if getattr(spec, "host_only", False) else nat.value("ion_sh_max_n_r_" + suffix)
        if spec.r_points > maxr:
            raise exceptions.UnsupportedMesh(f"r_points {spec.r_points} exceeds the device limit {maxr}")
        tb = self.operators.device_tables(self)
        mask = spec.mask(r=self.r)
        mask = None if np.isscalar(mask) and mask == 1 else np.asarray(mask, dtype=np.float64) * np.ones(len(self.r))
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        if hamiltonian and len(times) > 2 and np.ptp(self._tau_host[1:]) > 1e-12 * abs(self._tau_host[1]):
            # the coupled-line spikes are built for one tau
            raise exceptions.UnsupportedMesh("kinetic_energy_derivation='hamiltonian' needs a uniform time step")
        efield = np.zeros(len(times))
        gauge, h2r, rq = nat.ION_GAUGE_LENGTH, None, tb["rq"]
        if isinstance(self.operators, mo.SphericalHarmonicVelocityGaugeOperators):
            # the velocity-gauge operators take A at the step's own time
            # (times_to_current, sims.py:195-196); the tables carry its factors
            gauge = nat.ION_GAUGE_VELOCITY
            vt = self.operators.velocity_tables(self)
            rq, h2r = vt["rq"], vt["h2r"]
            efield[1:] = potentials.vector_potential_table(spec.electric_potential, times)[1:]
        else:
            efield[1:] = np.asarray(
                spec.electric_potential.get_electric_field_amplitude(times[1:] + (spec.time_step / 2)), np.float64
            ) * np.ones(len(times) - 1)
        sl, sg = [], []
        for s in spec.test_states:
            comps = list(s)
            if len(comps) != 1:
                raise exceptions.UnsupportedMesh("device inner products need single-l test states")
            sl.append(comps[0].l)
            sg.append(self.get_radial_g_for_state(comps[0]) * 1)
        # the initial psi as its component rows (only they are uploaded); the
        # full (l, r) array is formed if something reads it
        g0_rows, g0_vals = self._g_rows_for_state(spec.initial_state)
        shape = self.mesh_shape

        def full_g0():
            g = np.zeros(shape, dtype=np.complex128)
            for l, v in zip(g0_rows, g0_vals):
                g[l, :] = v
            return g

        self.tables = dev.ShTables(
            n_r=spec.r_points, n_l=spec.l_bound, hd=tb["hd"], hoff=tb["hoff"], rq=rq, cl=tb["cl"], mask=mask,
            tau=self._tau_host.copy(), efield=efield, kinv=tb["kinv"], cent=tb["cent"], corr0=tb["corr0"],
            state_l=sl, state_g=_radial_states_array(sg, spec.r_points),
            weight=self.inner_product_multiplier, g0=core.LazyArray(full_g0), t0=0, t_final=len(times) - 1,
            g0_rows=np.asarray(g0_rows, dtype=np.int64),
            g0_row_data=np.array(g0_vals, dtype=np.complex128).reshape(len(g0_rows), spec.r_points),
            store_every=spec.store_data_every, gauge=gauge, h2r=h2r, hcross=tb.get("cross"),
        )
        if getattr(spec, "host_only", False):
            return
        self._dsim = dev.ShDeviceSim(self.tables, self.precision)
        self._batch = dev.ShBatch(self.precision, [self._dsim])

    def _init_device_adi(self):
        """AlternatingDirectionImplicit over total_hamiltonian
        (evolution_methods.py:46-77, mesh_operators.py:1020-1035): per step
        E(H0), I(H_int), E(H_int), I(H0), then the mask, with H0 the radial
        Hamiltonian of each l and H_int = c_l (-q r_j) E(t + dt/2) between
        l-neighbours at each r.  That is the cylindrical ADI step on the same
        C-order layout with z = l (strided) and rho = r (contiguous), so it
        runs on that kernel pair (complex128)."""
        spec, sim = self.spec, self.sim
        if isinstance(self.operators, mo.SphericalHarmonicVelocityGaugeOperators):
            raise exceptions.UnsupportedMesh("the velocity gauge's h2 is not tridiagonal: no ADI device path")
        _adi_precision(self, "spherical-harmonic ADI")
        self._adi = True
        self.fused_data = False
        nr, L = spec.r_points, spec.l_bound
        cap = _adi_cap(self)
        if nr > cap or L > cap:
            raise exceptions.UnsupportedMesh(f"mesh {L} x {nr} exceeds the ADI device limit {cap} per line")
        tb = self.operators.device_tables(self)
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        efield = np.zeros(len(times))
        efield[1:] = np.asarray(
            spec.electric_potential.get_electric_field_amplitude(times[1:] + (spec.time_step / 2)), np.float64
        ) * np.ones(len(times) - 1)
        mask = spec.mask(r=self.r)
        mask = None if np.isscalar(mask) and mask == 1 else np.broadcast_to(
            np.asarray(mask, dtype=np.float64) * np.ones(nr), (L, nr)).copy()
        g0 = self.get_g_for_state(spec.initial_state)
        test_g = np.array([self.get_g_for_state(s).reshape(-1) for s in spec.test_states], dtype=np.complex128)
        arrays = dict(hz_d=None, hz_off=np.asarray(tb["cl"][: L - 1], dtype=np.float64), hr_d=tb["hd"],
                      hr_off=tb["hoff"], zq=None, tau=self._tau_host, efield=efield, mask=mask,
                      hz_off_col=tb["rq"])
        self.tables = dict(arrays, g0=g0, state_g=test_g)
        if getattr(spec, "host_only", False):
            return
        self._adi_setup(L, nr, arrays, g0, test_g)

    def _psi_device(self):
        return self._g if self._adi else self._dsim.g

    def _psi_residual(self):
        return None if self._adi else self._dsim.g_lo

    def _sh_observables(self, radii=()):
        """(<r>, <z>, norm by l, norm within radii) in one device pass."""
        import torch

        radii = tuple(radii)
        if len(radii) > 8:
            head = self._sh_observables(radii[:8])
            return head[0], head[1], head[2], list(head[3]) + list(self._sh_observables(radii[8:])[3])
        if not hasattr(self, "_d_obs_tables"):
            cl = np.asarray(self.operators.c_l(np.arange(self.spec.l_bound)), dtype=np.float64)
            self._d_obs_tables = (dev.to_dev(np.asarray(self.r, dtype=np.float64)), dev.to_dev(cl))
        d_r, d_cl = self._d_obs_tables
        g = self._psi_device()
        lo = self._psi_residual()
        nr, nl = self.spec.r_points, self.spec.l_bound
        d_radii = dev.to_dev(np.asarray(radii if radii else [0.0], dtype=np.float64))
        nbytes = nat.value("ion_sh_observables_scratch_bytes", nr, nl, len(radii))
        scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=g.device)
        res = torch.empty(2 + nl + len(radii), dtype=torch.float64, device=g.device)
        w = float(self.inner_product_multiplier)
        if g.dtype == torch.complex128:
            nat.call("ion_sh_observables_c128", dev.ptr(g), nr, nl, dev.ptr(d_r), dev.ptr(d_cl), len(radii),
                     dev.ptr(d_radii), w, dev.ptr(res), dev.ptr(scratch), int(nbytes), dev.stream_ptr())
        else:
            nat.call("ion_sh_observables_c64", dev.ptr(g), dev.ptr(lo), nr, nl, dev.ptr(d_r), dev.ptr(d_cl),
                     len(radii), dev.ptr(d_radii), w, dev.ptr(res), dev.ptr(scratch), int(nbytes), dev.stream_ptr())
        v = res.cpu().numpy()
        return float(v[0]), float(v[1]), v[2:2 + nl].copy(), v[2 + nl:].tolist()

    def z_expectation_value(self):
        """<z>: the F-order dipole operator (mesh_operators.py:1086-1104)."""
        return self._sh_observables()[1]

    def _energy_operators(self):
        """H0: the radial Hamiltonian of each l (hd, hoff: the Lagrangian
        kinetic energy, the internal potential and the l = 0 correction,
        mesh_operators.py:889-928, 244-269) along r; the interaction per unit
        field: c_l (-q r_j) between l-neighbours at each r times
        E(t + dt/2) (interaction_hamiltonian, mesh_operators.py:988-1018).
        The velocity gauge's interaction couples (l, r) with (l+1, r +- 1)
        as well: the device has no form of it (the reference's own total
        energy in that gauge raises: its interaction operators are bare
        sparse matrices that SumOfOperators.apply cannot apply)."""
        tb = self.operators.device_tables(self)
        L, nr = self.spec.l_bound, self.spec.r_points
        internal = (np.asarray(tb["hd"], dtype=np.float64).reshape(L, nr), np.append(tb["hoff"], 0.0), None, 0)
        if tb.get("cross") is not None:  # the Hamiltonian-derived kinetic energy joins consecutive lines
            internal = (internal[0], np.append(tb["hoff"], tb["cross"]), None, nat.ION_HOP_WRAP_B)
        if isinstance(self.operators, mo.SphericalHarmonicVelocityGaugeOperators):
            return (L, nr), internal, "unsupported", None
        cl = np.append(np.asarray(tb["cl"], dtype=np.float64)[: L - 1], 0.0)
        inter = (None, None, np.outer(cl, np.asarray(tb["rq"], dtype=np.float64)), 0)
        spec, sim = self.spec, self.sim
        return (L, nr), internal, inter, lambda: float(
            spec.electric_potential.get_electric_field_amplitude(sim.time + spec.time_step / 2))

    def radial_probability_current(self):
        """(z > 0, z < 0): the radial probability current through each shell
        r_j, as DirectionalRadialProbabilityCurrent.store forms it
        (data.py:467-505) from get_radial_probability_current_density_mesh__
        spatial (meshes.py:1358-1371): the r-current operator of
        r_probability_current__spatial (mesh_operators.py:1107-1127) on psi
        rebuilt on the theta_calc grid (theta_points from 0 to pi,
        meshes.py:1456-1458, 1497-1517), Im(conj(psi) G psi) sin(theta)
        dtheta 2 pi summed over each hemisphere (theta <= pi/2 is z > 0),
        times r_j^2.  On the device the theta sum is folded into l-pair
        weights (ion_sh_radial_current_*)."""
        import torch

        if getattr(self, "_d_current", None) is None:
            spec = self.spec
            nr, L = spec.r_points, spec.l_bound
            theta = np.linspace(0, np.pi, int(spec.theta_points))
            ylm = sph_harm_m0(np.arange(L), theta)  # (L, n_theta)
            wt = u.twopi * np.abs(theta[1] - theta[0]) * np.sin(theta)
            up = theta <= np.pi / 2
            w_pos = (ylm[:, up] * wt[up]) @ ylm[:, up].T
            w_neg = (ylm[:, ~up] * wt[~up]) @ ylm[:, ~up].T
            j = np.arange(1, nr, dtype=np.float64)
            od = (u.hbar / (2 * spec.test_mass * self.delta_r ** 3)) / (j ** 2 - 0.25)
            self._d_current = tuple(dev.to_dev(np.ascontiguousarray(a, dtype=np.float64))
                                    for a in (od, self.r, w_pos, w_neg))
        d_od, d_r, d_wp, d_wn = self._d_current
        g = self._psi_device()
        lo = self._psi_residual()
        nr, L = self.spec.r_points, self.spec.l_bound
        out = torch.empty(2 * nr, dtype=torch.float64, device=g.device)
        if g.dtype == torch.complex128:
            nat.call("ion_sh_radial_current_c128", dev.ptr(g), nr, L, dev.ptr(d_od), dev.ptr(d_r), dev.ptr(d_wp),
                     dev.ptr(d_wn), dev.ptr(out), dev.stream_ptr())
        else:
            nat.call("ion_sh_radial_current_c64", dev.ptr(g), dev.ptr(lo), nr, L, dev.ptr(d_od), dev.ptr(d_r),
                     dev.ptr(d_wp), dev.ptr(d_wn), dev.ptr(out), dev.stream_ptr())
        v = out.cpu().numpy()
        return v[:nr].copy(), v[nr:].copy()

    def r_expectation_value(self):
        return self._sh_observables()[0]

    def norm_by_l(self):
        """SphericalHarmonicMesh.norm_by_l (meshes.py:1133-1136)."""
        return self._sh_observables()[2]

    def norm_within_radius(self, radii):
        return self._sh_observables(radii)[3]

    def _tau_dev(self):
        return self._d["tau"] if self._adi else self._dsim.d_tau

    def _evolve_steps(self, n):
        if self._adi:
            self._adi_evolve_steps(n)
        else:
            self._batch.run(n)

    def _reduce_current(self):
        if self._adi:
            self._adi_reduce_current()
        else:
            self._batch.reduce()

    def _pull_data(self):
        return self._adi_pull_data() if self._adi else self._dsim.data()


# ==========================================================================
# spherical slice
# ==========================================================================


class SphericalSliceMesh(_AdiDevice, QuantumMesh):
    """SphericalSliceMesh (meshes.py:887-983): g = sqrt(2 pi sin theta) r psi
    on (r, theta), theta contiguous.  Under AlternatingDirectionImplicit each
    step is E(H_theta), I(H_r), E(H_r), I(H_theta), then the mask, on the
    two-direction ADI kernels with r strided (implicit first) and theta
    contiguous.  The device holds psi' = D^-1 g, D the diagonal in theta that
    symmetrises the theta operator (SphericalSliceLengthGaugeOperators.
    device_tables); g, the norms and the overlaps are formed with D."""

    mesh_storage_method = ("r", "theta")

    def __init__(self, sim):
        super().__init__(sim)
        self.r = np.linspace(0, self.spec.r_bound, self.spec.r_points)
        self.theta = np.delete(np.linspace(0, u.pi, self.spec.theta_points + 1), 0)
        self.delta_r = self.r[1] - self.r[0]
        self.delta_theta = self.theta[1] - self.theta[0]
        self.inner_product_multiplier = self.delta_r * self.delta_theta
        self.r = self.r + self.delta_r / 2
        self.theta = self.theta - self.delta_theta / 2
        self.r_max = np.max(self.r)
        self.r_mesh, self.theta_mesh = np.meshgrid(self.r, self.theta, indexing="ij")
        self.mesh_points = len(self.r) * len(self.theta)
        self.mesh_shape = np.shape(self.r_mesh)
        self._state_g_cache = {}
        self._init_device()

    @property
    def z_mesh(self):
        return self.r_mesh * np.cos(self.theta_mesh)

    @property
    def g_factor(self):
        return np.sqrt(u.twopi * np.sin(self.theta_mesh)) * self.r_mesh

    def wrapping_direction_to_order(self, wrapping_direction):
        if wrapping_direction is None:
            return None
        if wrapping_direction == WrappingDirection.R:
            return "F"
        if wrapping_direction == WrappingDirection.THETA:
            return "C"
        raise ValueError(f"{wrapping_direction} is not a valid specifier for flatten_mesh (valid specifiers: 'r', 'theta')")

    def get_g_for_state(self, state):
        """meshes.py:961-967."""
        if state in self._state_g_cache:
            return self._state_g_cache[state]
        g = self.g_factor * state(self.r_mesh, self.theta_mesh, 0)
        g = np.asarray(g, dtype=np.complex128)
        g = g / np.sqrt(np.sum(np.conj(g) * g).real * self.inner_product_multiplier)
        g = g * state.amplitude
        self._state_g_cache[state] = g
        return g

    def _init_device(self):
        spec, sim = self.spec, self.sim
        if not isinstance(self.operators, mo.SphericalSliceLengthGaugeOperators):
            raise exceptions.UnsupportedMesh(f"{type(self.operators).__name__} has no device path on SphericalSliceMesh")
        if not isinstance(spec.evolution_method, em.AlternatingDirectionImplicit):
            raise exceptions.UnsupportedMesh(
                f"{type(spec.evolution_method).__name__} has no device path on SphericalSliceMesh")
        if self.precision != core.Precision.C128:
            # it evolves g / D, D the similarity scaling that makes the theta
            # operator symmetric and that spans orders of magnitude across
            # theta; FP32 sweeps of the scaled state lose ~1e-5 in the
            # populations within a few hundred steps
            raise exceptions.UnsupportedMesh("the spherical-slice device path is complex128")
        cap = _adi_cap(self)
        if spec.r_points > cap or spec.theta_points > cap:
            raise exceptions.UnsupportedMesh(f"mesh {spec.r_points} x {spec.theta_points} exceeds {cap} points per line")
        tb = self.operators.device_tables(self)
        self._D = np.asarray(tb["d"], dtype=np.float64)[None, :] * np.ones(self.mesh_shape)
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        efield = np.zeros(len(times))
        efield[1:] = np.asarray(spec.electric_potential.get_electric_field_amplitude(times[1:]), np.float64) * np.ones(len(times) - 1)
        mask = spec.mask(r=self.r_mesh)
        mask = None if np.isscalar(mask) and mask == 1 else np.asarray(mask, np.float64) * np.ones(self.mesh_shape)
        g0 = self.get_g_for_state(spec.initial_state)
        # overlaps of g = D psi' are those of psi' with D s
        test_g = np.array([(self.get_g_for_state(s) * self._D).reshape(-1) for s in spec.test_states],
                          dtype=np.complex128)
        arrays = dict(hz_d=tb["hz_d"], hz_off=tb["hz_off"], hr_d=tb["hr_d"], hr_off=tb["hr_off"], zq=None,
                      tau=self._tau_host, efield=efield, mask=mask, hz_off_col=None, hr_off_row=tb["hr_off_row"],
                      zq_pt=tb["zq_pt"])
        self.tables = dict(arrays, g0=g0, state_g=test_g, d=tb["d"])
        if getattr(spec, "host_only", False):
            return
        self._adi_setup(spec.r_points, spec.theta_points, arrays, g0 / self._D, test_g)
        self._d_w2 = dev.to_dev((self._D ** 2).reshape(1, -1))
        self._d_norm_scratch = torch.empty(1, dtype=torch.float64, device=dev.device())

    @property
    def g(self) -> np.ndarray:
        return self._psi_device().cpu().numpy().astype(np.complex128).reshape(self.mesh_shape) * self._D

    @g.setter
    def g(self, value):
        v = np.asarray(value, dtype=np.complex128).reshape(self.mesh_shape) / self._D
        self._g.copy_(torch.from_numpy(np.ascontiguousarray(v)).to(self._g.device, self._g.dtype))

    def _weighted_norms(self, weights):
        return super()._weighted_norms([np.asarray(w, dtype=np.float64) * self._D ** 2 for w in weights])

    def _psi_device(self):
        return self._g

    def _tau_dev(self):
        return self._d["tau"]

    def _evolve_steps(self, n):
        self._adi_evolve_steps(n)

    def _reduce_current(self):
        """Overlaps through the reducer (states scaled by D); the norm with
        the weights D^2."""
        tf = len(self.sim.times) - 1
        slot = dev.data_slot(self._t, tf, self.spec.store_data_every)
        self._reducer(self._g, self._d_norm_scratch, self._d_ip[slot])
        n = self.mesh_points
        nbytes = nat.value("ion_weighted_norms_scratch_bytes", n, 1)
        if not hasattr(self, "_d_wn_scratch") or self._d_wn_scratch.numel() * 8 < nbytes:
            self._d_wn_scratch = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=dev.device())
        args = (1, dev.ptr(self._d_w2), float(self.inner_product_multiplier), dev.ptr(self._d_norm[slot:slot + 1]),
                dev.ptr(self._d_wn_scratch), int(nbytes), dev.stream_ptr())
        if self._g.dtype == torch.complex128:
            nat.call("ion_weighted_norms_c128", n, dev.ptr(self._g), *args)
        else:
            nat.call("ion_weighted_norms_c64", n, dev.ptr(self._g), None, *args)

    def _pull_data(self):
        return self._adi_pull_data()


# ==========================================================================
# rectangle
# ==========================================================================


class RectangleMesh(_AdiDevice, QuantumMesh):
    """RectangleMesh (meshes.py:430-506): psi on (z, x), x contiguous.  Under
    AlternatingDirectionImplicit each step is E(H_z), I(H_x), E(H_x), I(H_z),
    then the mask: the two-direction ADI kernel pair with z strided, x
    contiguous, the contiguous pass first (complex128)."""

    mesh_storage_method = ("z", "x")

    def __init__(self, sim):
        super().__init__(sim)
        self.z = np.linspace(-self.spec.z_bound, self.spec.z_bound, self.spec.z_points)
        self.x = np.linspace(-self.spec.x_bound, self.spec.x_bound, self.spec.x_points)
        self.delta_z = np.abs(self.z[1] - self.z[0])
        self.delta_x = np.abs(self.x[1] - self.x[0])
        self.inner_product_multiplier = self.delta_z * self.delta_x
        self.g_factor = 1
        self.z_center_index = int(self.spec.z_points // 2)
        self.x_center_index = int(self.spec.x_points // 2)
        self.z_mesh, self.x_mesh = np.meshgrid(self.z, self.x, indexing="ij")
        self.r_mesh = np.sqrt((self.z_mesh ** 2) + (self.x_mesh ** 2))
        self.mesh_points = len(self.z) * len(self.x)
        self.mesh_shape = np.shape(self.r_mesh)
        self._state_g_cache = {}
        self._init_device()

    @property
    def theta_mesh(self):
        return np.arctan2(self.x_mesh, self.z_mesh)

    def wrapping_direction_to_order(self, wrapping_direction):
        if wrapping_direction is None:
            return None
        if wrapping_direction == WrappingDirection.Z:
            return "F"
        if wrapping_direction == WrappingDirection.X:
            return "C"
        raise ValueError(f"{wrapping_direction} is not a valid specifier for flatten_mesh (valid specifiers: 'z', 'x')")

    def get_g_for_state(self, state):
        """meshes.py:487-493."""
        if state in self._state_g_cache:
            return self._state_g_cache[state]
        g = np.asarray(state(self.r_mesh, self.theta_mesh), dtype=np.complex128)
        g = g / np.sqrt(np.sum(np.conj(g) * g).real * self.inner_product_multiplier)
        g = g * state.amplitude
        self._state_g_cache[state] = g
        return g

    def _init_device(self):
        spec, sim = self.spec, self.sim
        if not isinstance(self.operators, mo.RectangleLengthGaugeOperators):
            raise exceptions.UnsupportedMesh(f"{type(self.operators).__name__} has no device path on RectangleMesh")
        if not isinstance(spec.evolution_method, em.AlternatingDirectionImplicit):
            raise exceptions.UnsupportedMesh(f"{type(spec.evolution_method).__name__} has no device path on RectangleMesh")
        _adi_precision(self, "rectangle")
        cap = _adi_cap(self)
        if spec.z_points > cap or spec.x_points > cap:
            raise exceptions.UnsupportedMesh(f"mesh {spec.z_points} x {spec.x_points} exceeds {cap} points per line")
        tb = self.operators.device_tables(self)
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        efield = np.zeros(len(times))
        efield[1:] = np.asarray(spec.electric_potential.get_electric_field_amplitude(times[1:]), np.float64) * np.ones(len(times) - 1)
        mask = spec.mask(r=self.r_mesh)
        mask = None if np.isscalar(mask) and mask == 1 else np.asarray(mask, np.float64) * np.ones(self.mesh_shape)
        g0 = self.get_g_for_state(spec.initial_state)
        test_g = np.array([self.get_g_for_state(s).reshape(-1) for s in spec.test_states], dtype=np.complex128)
        arrays = dict(hz_d=tb["hz_d"], hz_off=tb["hz_off"], hr_d=tb["hr_d"], hr_off=tb["hr_off"], zq=tb["zq"],
                      tau=self._tau_host, efield=efield, mask=mask, hz_off_col=None)
        self.tables = dict(arrays, g0=g0, state_g=test_g)
        if getattr(spec, "host_only", False):
            return
        self._adi_setup(spec.z_points, spec.x_points, arrays, g0, test_g)
        self._cm.order = nat.ION_ADI_CONTIG_FIRST

    def _energy_operators(self):
        return _two_axis_energy_operators(self, self.spec.z_points, self.spec.x_points)

    def _psi_device(self):
        return self._g

    def _tau_dev(self):
        return self._d["tau"]

    def _evolve_steps(self, n):
        self._adi_evolve_steps(n)

    def _reduce_current(self):
        self._adi_reduce_current()

    def _pull_data(self):
        return self._adi_pull_data()


# ==========================================================================
# cylindrical slice
# ==========================================================================


class CylindricalSliceMesh(_AdiDevice, QuantumMesh):
    mesh_storage_method = ("z", "rho")

    def __init__(self, sim):
        super().__init__(sim)
        self.z = np.linspace(-self.spec.z_bound, self.spec.z_bound, self.spec.z_points)
        self.rho = np.delete(np.linspace(0, self.spec.rho_bound, self.spec.rho_points + 1), 0)
        self.delta_z = self.z[1] - self.z[0]
        self.delta_rho = self.rho[1] - self.rho[0]
        self.inner_product_multiplier = self.delta_z * self.delta_rho
        self.rho = self.rho - self.delta_rho / 2
        self.z_center_index = int(self.spec.z_points // 2)
        self.z_mesh, self.rho_mesh = np.meshgrid(self.z, self.rho, indexing="ij")
        self.r_mesh = np.sqrt((self.z_mesh ** 2) + (self.rho_mesh ** 2))
        self.mesh_points = len(self.z) * len(self.rho)
        self.mesh_shape = np.shape(self.r_mesh)
        self._state_g_cache = {}
        self._init_device()

    @property
    def g_factor(self):
        return np.sqrt(u.twopi * self.rho_mesh)

    @property
    def theta_mesh(self):
        return np.arccos(self.z_mesh / self.r_mesh)

    def wrapping_direction_to_order(self, wrapping_direction):
        if wrapping_direction is None:
            return None
        if wrapping_direction == WrappingDirection.Z:
            return "F"
        if wrapping_direction == WrappingDirection.RHO:
            return "C"
        raise ValueError(f"{wrapping_direction} is not a valid specifier for flatten_mesh (valid specifiers: 'z', 'rho')")

    def get_g_for_state(self, state):
        """meshes.py:601-607."""
        if state in self._state_g_cache:
            return self._state_g_cache[state]
        g = self.g_factor * state(self.r_mesh, self.theta_mesh, 0)
        g = g / np.sqrt(np.sum(np.conj(g) * g).real * self.inner_product_multiplier)
        g = g * state.amplitude
        g = np.asarray(g, dtype=np.complex128)
        self._state_g_cache[state] = g
        return g

    def _init_device(self):
        spec, sim = self.spec, self.sim
        if not isinstance(self.operators, mo.CylindricalSliceLengthGaugeOperators):
            raise exceptions.UnsupportedMesh(f"{type(self.operators).__name__} has no device path on CylindricalSliceMesh")
        if not isinstance(spec.evolution_method, em.AlternatingDirectionImplicit):
            raise exceptions.UnsupportedMesh(
                f"{type(spec.evolution_method).__name__} has no device path on CylindricalSliceMesh"
            )
        _adi_precision(self, "cylindrical")
        tb = self.operators.device_tables(self)
        times = sim.times
        self._tau_host = np.zeros(len(times))
        self._tau_host[1:] = (times[1:] - times[:-1]) / (2 * u.hbar)
        efield = np.zeros(len(times))
        efield[1:] = np.asarray(spec.electric_potential.get_electric_field_amplitude(times[1:]), np.float64) * np.ones(len(times) - 1)
        mask = spec.mask(r=self.r_mesh)
        mask = None if np.isscalar(mask) and mask == 1 else np.asarray(mask, np.float64) * np.ones(self.mesh_shape)
        g0 = self.get_g_for_state(spec.initial_state)
        test_g = np.array([self.get_g_for_state(s).reshape(-1) for s in spec.test_states], dtype=np.complex128)
        self.tables = dict(tb, mask=mask, tau=self._tau_host.copy(), efield=efield, g0=g0, state_g=test_g)
        if getattr(spec, "host_only", False):
            return
        self._adi_setup(spec.z_points, spec.rho_points, dict(
            hz_d=tb["hz_d"], hz_off=tb["hz_off"], hr_d=tb["hr_d"], hr_off=tb["hr_off"], zq=tb["zq"],
            tau=self._tau_host, efield=efield, mask=mask, hz_off_col=None), g0, test_g)

    def _energy_operators(self):
        return _two_axis_energy_operators(self, self.spec.z_points, self.spec.rho_points)

    def _psi_device(self):
        return self._g

    def _tau_dev(self):
        return self._d["tau"]

    def _evolve_steps(self, n):
        self._adi_evolve_steps(n)

    def _reduce_current(self):
        self._adi_reduce_current()

    def _pull_data(self):
        return self._adi_pull_data()
