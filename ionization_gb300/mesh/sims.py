"""Specifications and simulations: the spec -> ``to_sim()`` -> ``run()`` API.

Keeps the reference's surface (ionization/mesh/sims.py:36-1094): the same
specification classes and keyword arguments, ``MeshSimulation.run`` with
``progress_bar`` / ``callback`` / ``checkpoint_callback``, the time grid, the
data times and ``sim.data``.  One extra keyword, ``precision`` ("c128" by
default, or "c64"), selects the device arithmetic of the wavefunction.

``run`` advances the device-resident wavefunction in segments: without a
callback a segment runs to the next point where the host has to act (a data
time of a mesh without fused reductions, a checkpoint, the end); with a
callback every step is its own segment, as in the reference loop.
"""

import datetime
import logging
import os
import pickle
from copy import deepcopy

import numpy as np

from .. import core, exceptions, potentials, states
from .. import units as u
from . import data, evolution_methods, mesh_operators, meshes

logger = logging.getLogger(__name__)


class MeshSimulation:
    def __init__(self, spec):
        self.spec = spec
        self.name = spec.name
        self.status = "initialized"
        self.latest_checkpoint_time = datetime.datetime.now(datetime.timezone.utc)
        self.times = self.get_times()
        self.time_index = 0
        self.data_time_index = 0
        self.time_steps = len(self.times)

        self.mesh = self.spec.mesh_type(self)

        idx = np.arange(self.time_steps)
        self.data_mask = np.equal(idx, 0) + np.equal(idx, self.time_steps - 1)
        if self.spec.store_data_every >= 1:
            self.data_mask += np.equal(idx % self.spec.store_data_every, 0)
        self.data_times = self.times[self.data_mask]
        self.data_indices = idx[self.data_mask]
        self.data_time_steps = len(self.data_times)
        self.spacetime_points = self.time_steps * self.mesh.mesh_points

        self.data = data.Data(self)
        self.datastores_by_type = {ds.__class__: deepcopy(ds) for ds in self.spec.datastores}
        for ds in self.datastores_by_type.values():
            ds.init(self)
        self.warnings = {}
        self._initial_data_done = False

    def __repr__(self):
        return f"{self.__class__.__name__}({self.name})"

    @property
    def time(self):
        return self.times[self.time_index]

    @property
    def times_to_current(self):
        return self.times[: self.time_index + 1]

    def get_times(self):
        """sims.py:198-220 (fixed time step)."""
        if callable(self.spec.time_step):
            raise exceptions.UnsupportedMesh("callable time steps have no device path")
        total = self.spec.time_final - self.spec.time_initial
        return np.linspace(self.spec.time_initial, self.spec.time_final, int(total / self.spec.time_step) + 1)

    def get_blank_data(self, dtype=np.float64):
        a = np.empty(self.data_time_steps, dtype=dtype)
        a.fill(np.nan)
        return a

    @property
    def percent_completed(self):
        return round(100 * self.time_index / max(self.time_steps - 1, 1), 2)

    # ---- data ----
    def _pull_data(self):
        norm, ips = self.mesh._pull_data()
        for ds in self.datastores_by_type.values():
            ds.pull(norm, ips)
        self._check_norms()

    def _check_norms(self):
        """Norm-growth warnings of MeshSimulation.check (sims.py:228-240)."""
        if data.Norm not in self.datastores_by_type:
            return
        n = self.data.norm
        for k in range(1, self.data_time_steps):
            if np.isnan(n[k]):
                break
            if n[k] > 1.001 * n[0] or n[k] > 1.001 * n[k - 1]:
                msg = f"Wavefunction norm ({n[k]}) grew by more than 0.1% at data index {k} for {self}"
                self.warnings.setdefault("norm_growth", []).append(core.WarningRecord(k, msg))

    @property
    def _stores_at_data_times(self):
        return [ds for ds in self.datastores_by_type.values() if ds.stores_at_data_times]

    def _store_data_time(self):
        """Datastores that read the wavefunction at a data time."""
        if self.data_mask[self.time_index]:
            self.data_time_index = int(np.sum(self.data_indices < self.time_index))
            for ds in self._stores_at_data_times:
                ds.store()

    def _next_stop(self, callback_given):
        last = self.time_steps - 1
        if callback_given:
            return self.time_index + 1
        if not self.mesh.fused_data or self._stores_at_data_times:
            later = self.data_indices[self.data_indices > self.time_index]
            return int(later[0]) if len(later) else last
        return last

    def run(self, progress_bar: bool = False, callback=None, checkpoint_callback=None, max_steps=None):
        """Evolve from the current time index to the end (sims.py:255-346).

        ``max_steps`` bounds the number of steps of this call (the run can be
        resumed by calling ``run`` again)."""
        last = self.time_steps - 1
        if not self._initial_data_done:
            self.mesh._reduce_current()  # data of time index 0
            self._store_data_time()
            self._initial_data_done = True
        if callback is not None:
            callback(self)
        stop_at = last if max_steps is None else min(last, self.time_index + int(max_steps))
        self.status = "running"
        while self.time_index < stop_at:
            nxt = min(self._next_stop(callback is not None), stop_at)
            n = nxt - self.time_index
            self.mesh._evolve_steps(n)
            self.time_index = nxt
            if not self.mesh.fused_data and self.data_mask[self.time_index]:
                self.mesh._reduce_current()
            self._store_data_time()
            if callback is not None:
                self._pull_data()
                callback(self)
            if self.spec.checkpoints:
                now = datetime.datetime.now(datetime.timezone.utc)
                if (now - self.latest_checkpoint_time) > self.spec.checkpoint_every:
                    self.do_checkpoint(now, checkpoint_callback)
        self._pull_data()
        self.data_time_index = int(np.sum(self.data_indices <= self.time_index))
        self.status = "finished" if self.time_index == last else "paused"

    def do_checkpoint(self, now, callback=None):
        path = self.save(target_dir=self.spec.checkpoint_dir, save_mesh=True)
        if callback is not None:
            callback(path)
        self.latest_checkpoint_time = now

    # ---- persistence (sims.py:405-438): psi is copied to the host ----
    def save(self, target_dir=None, save_mesh: bool = True):
        target_dir = target_dir or os.getcwd()
        path = os.path.join(target_dir, f"{self.name}.sim")
        if self.mesh is not None:  # a simulation whose mesh was dropped keeps its data as they are
            self._pull_data()
        keep = save_mesh and self.mesh is not None
        # ``native``: the device arrays as they are, so a reload continues the
        # run bit for bit whatever transform lies between them and ``g``
        state = dict(spec=self.spec, time_index=self.time_index, g=self.mesh.g if keep else None,
                     native=self.mesh._native_state() if keep else None,
                     initial_data_done=self._initial_data_done,
                     data={type(ds): vars(ds).copy() for ds in self.datastores_by_type.values()})
        for d in state["data"].values():
            d.pop("sim", None)
            d.pop("spec", None)
        tmp = path + ".tmp"
        with open(tmp, "wb") as f:
            pickle.dump(state, f)
        os.replace(tmp, path)
        return path

    @classmethod
    def load(cls, path):
        """Rebuild the simulation and restore psi, the time index and data."""
        with open(path, "rb") as f:
            state = pickle.load(f)
        sim = state["spec"].to_sim()
        if state["g"] is not None:
            if state.get("native") is not None:
                sim.mesh._set_native_state(state["native"])
            else:
                sim.mesh.g = state["g"]
            sim._restore_index(state["time_index"])
        else:
            sim.mesh = None
        for typ, vals in state["data"].items():
            ds = sim.datastores_by_type.get(typ)
            if ds is None:
                continue
            for k, v in vals.items():
                cur = getattr(ds, k, None)
                if isinstance(cur, np.ndarray):
                    cur[...] = v
                elif isinstance(cur, dict):
                    for kk in cur:
                        cur[kk][...] = v[kk]
        sim._initial_data_done = state["initial_data_done"]
        return sim

    def _restore_index(self, t):
        self.time_index = int(t)
        m = self.mesh
        if hasattr(m, "_dsim"):
            m._dsim.t = int(t)
            m._batch.invalidate()
        else:
            m._t = int(t)

    def info(self):
        return f"{self.__class__.__name__}({self.name}): {self.mesh.__class__.__name__}, {self.time_steps} times"


class SphericalHarmonicSimulation(MeshSimulation):
    """Adds the top-l norm check of sims.py:979-990."""

    def _check_norms(self):
        super()._check_norms()
        g_top = self.mesh.g[-1]
        norm_top = np.sum(np.abs(g_top) ** 2) * self.mesh.inner_product_multiplier
        if norm_top > 1e-6:
            msg = f"Wavefunction norm in largest angular momentum state is large at time index {self.time_index}"
            self.warnings.setdefault("norm_in_largest_l", []).append(core.WarningRecord(self.time_index, msg))


class MeshSpecification:
    simulation_type = MeshSimulation
    mesh_type = meshes.QuantumMesh

    def __init__(
        self,
        name: str,
        test_mass: float = u.electron_mass_reduced,
        test_charge: float = u.electron_charge,
        initial_state=states.HydrogenBoundState(1, 0),
        test_states=tuple(),
        internal_potential=potentials.CoulombPotential(charge=u.proton_charge),
        electric_potential=potentials.NoElectricPotential(),
        electric_potential_dc_correction: bool = False,
        electric_potential_fluence_correction: bool = False,
        mask=potentials.NoMask(),
        operators=None,
        evolution_method=None,
        time_initial: float = 0 * u.asec,
        time_final: float = 200 * u.asec,
        time_step: float = 1 * u.asec,
        checkpoints: bool = False,
        checkpoint_every: datetime.timedelta = datetime.timedelta(hours=1),
        checkpoint_dir=None,
        animators=tuple(),
        store_data_every: int = 1,
        snapshot_times=(),
        snapshot_indices=(),
        snapshot_type=None,
        snapshot_kwargs=None,
        datastores=None,
        precision: str = "c128",
        **kwargs,
    ):
        self.name = str(name)
        self.file_name = kwargs.pop("file_name", self.name)
        for k, v in kwargs.items():
            setattr(self, k, v)
        if electric_potential_dc_correction or electric_potential_fluence_correction:
            raise exceptions.UnsupportedMesh("field DC / fluence correction is not part of the device path")
        if len(tuple(animators)) or len(tuple(snapshot_times)) or len(tuple(snapshot_indices)):
            raise exceptions.UnsupportedMesh("animators and snapshots are not part of the device path")
        self.test_mass = test_mass
        self.test_charge = test_charge
        self.initial_state = initial_state
        self.test_states = sorted(test_states) if len(test_states) else []
        if len(self.test_states) == 0:
            self.test_states = [self.initial_state]
        self.internal_potential = internal_potential
        self.electric_potential = electric_potential
        self.electric_potential_dc_correction = electric_potential_dc_correction
        self.electric_potential_fluence_correction = electric_potential_fluence_correction
        self.mask = mask
        self.operators = operators
        self.evolution_method = evolution_method
        self.time_initial = time_initial
        self.time_final = time_final
        self.time_step = time_step
        self.checkpoints = checkpoints
        self.checkpoint_every = checkpoint_every
        self.checkpoint_dir = checkpoint_dir
        self.animators = ()
        self.store_data_every = int(store_data_every)
        self.snapshot_times, self.snapshot_indices = set(), set()
        self.snapshot_type, self.snapshot_kwargs = snapshot_type, snapshot_kwargs or {}
        self.precision = core.Precision(precision)
        if datastores is None:
            datastores = [ds_type() for ds_type in data.DEFAULT_DATASTORE_TYPES]
        self.datastores = datastores
        self.datastore_types = tuple(sorted({ds.__class__ for ds in datastores}, key=lambda d: d.__name__))
        if len(self.datastores) != len(self.datastore_types):
            raise exceptions.DuplicateDatastores("Cannot duplicate datastores")

    def to_sim(self):
        return self.simulation_type(self)

    def __repr__(self):
        return f"{self.__class__.__name__}({self.name})"


class LineSpecification(MeshSpecification):
    mesh_type = meshes.LineMesh

    def __init__(
        self,
        name,
        internal_potential=potentials.SoftCoulombPotential(),
        initial_state=states.GaussianState(),
        z_bound: float = 10 * u.nm,
        z_points: int = 2 ** 9,
        use_numeric_eigenstates: bool = False,
        number_of_numeric_eigenstates: int = 100,
        analytic_eigenstate_type=None,
        operators=mesh_operators.LineLengthGaugeOperators(),
        evolution_method=evolution_methods.AlternatingDirectionImplicit(),
        **kwargs,
    ):
        if use_numeric_eigenstates:
            raise exceptions.UnsupportedMesh("numeric eigenstates are not part of the device path")
        super().__init__(name, internal_potential=internal_potential, initial_state=initial_state,
                         operators=operators, evolution_method=evolution_method, **kwargs)
        self.z_bound = z_bound
        self.z_points = int(z_points)
        self.use_numeric_eigenstates = False
        self.number_of_numeric_eigenstates = number_of_numeric_eigenstates
        self.analytic_eigenstate_type = analytic_eigenstate_type


class SphericalHarmonicSpecification(MeshSpecification):
    simulation_type = SphericalHarmonicSimulation
    mesh_type = meshes.SphericalHarmonicMesh

    def __init__(
        self,
        name,
        r_bound: float = 100 * u.bohr_radius,
        r_points: int = 1000,
        l_bound: int = 300,
        theta_points: int = 180,
        operators=mesh_operators.SphericalHarmonicLengthGaugeOperators(),
        evolution_method=evolution_methods.SplitInteractionOperator(),
        use_numeric_eigenstates: bool = True,
        numeric_eigenstate_max_energy: float = 20 * u.eV,
        numeric_eigenstate_max_angular_momentum: int = 5,
        **kwargs,
    ):
        super().__init__(name, operators=operators, evolution_method=evolution_method, **kwargs)
        self.r_bound = r_bound
        self.r_points = int(r_points)
        self.l_bound = int(l_bound)
        self.spherical_harmonics = tuple(core.SphericalHarmonic(l, 0) for l in range(self.l_bound))
        self.theta_points = theta_points
        self.use_numeric_eigenstates = bool(use_numeric_eigenstates)
        self.numeric_eigenstate_max_angular_momentum = min(self.l_bound - 1, numeric_eigenstate_max_angular_momentum)
        self.numeric_eigenstate_max_energy = numeric_eigenstate_max_energy


class SphericalSliceSpecification(MeshSpecification):
    """sims.py:907-950."""

    mesh_type = meshes.SphericalSliceMesh

    def __init__(
        self,
        name,
        r_bound: float = 20 * u.bohr_radius,
        r_points: int = 2 ** 10,
        theta_points: int = 2 ** 10,
        operators=mesh_operators.SphericalSliceLengthGaugeOperators(),
        evolution_method=evolution_methods.AlternatingDirectionImplicit(),
        **kwargs,
    ):
        super().__init__(name, operators=operators, evolution_method=evolution_method, **kwargs)
        self.r_bound = r_bound
        self.r_points = int(r_points)
        self.theta_points = int(theta_points)


class RectangleSpecification(MeshSpecification):
    """sims.py:765-833."""

    mesh_type = meshes.RectangleMesh

    def __init__(
        self,
        name,
        internal_potential=potentials.NoPotentialEnergy(),
        initial_state=None,
        z_bound: float = 10 * u.nm,
        z_points: int = 2 ** 9,
        x_bound: float = 10 * u.nm,
        x_points: int = 2 ** 9,
        operators=mesh_operators.RectangleLengthGaugeOperators(),
        evolution_method=evolution_methods.AlternatingDirectionImplicit(),
        **kwargs,
    ):
        if initial_state is None:
            initial_state = states.TwoDGaussianWavepacket()
        super().__init__(name, internal_potential=internal_potential, initial_state=initial_state,
                         operators=operators, evolution_method=evolution_method, **kwargs)
        self.z_bound = z_bound
        self.z_points = int(z_points)
        self.x_bound = x_bound
        self.x_points = int(x_points)


class CylindricalSliceSpecification(MeshSpecification):
    mesh_type = meshes.CylindricalSliceMesh

    def __init__(
        self,
        name,
        z_bound: float = 20 * u.bohr_radius,
        rho_bound: float = 20 * u.bohr_radius,
        z_points: int = 2 ** 9,
        rho_points: int = 2 ** 8,
        operators=mesh_operators.CylindricalSliceLengthGaugeOperators(),
        evolution_method=evolution_methods.AlternatingDirectionImplicit(),
        **kwargs,
    ):
        super().__init__(name, operators=operators, evolution_method=evolution_method, **kwargs)
        self.z_bound = z_bound
        self.rho_bound = rho_bound
        self.z_points = int(z_points)
        self.rho_points = int(rho_points)
