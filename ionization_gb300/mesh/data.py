"""Datastores (ionization/mesh/data.py:14-530): Fields, Norm, InnerProducts,
ZExpectationValue, RExpectationValue, NormWithinRadius, NormBySphericalHarmonic,
InternalEnergyExpectationValue, TotalEnergyExpectationValue,
DirectionalRadialProbabilityCurrent.

Norm and InnerProducts are filled from the FP64 device reductions made at the
data times of the run (fused into the step kernels, or a reduction kernel at
the data time); ``Fields`` is evaluated on the host from the pulse.  The
position and energy expectation values, partial norms and radial currents
are device reductions of the current wavefunction launched at each data
time (``store``).  The attribute
names on ``sim.data`` are the reference's.
"""

import numpy as np

from .. import exceptions, potentials


class Data:
    def __init__(self, sim):
        self.sim = sim
        self.times = sim.data_times

    def __getattr__(self, item):
        if item.startswith("__") and item.endswith("__"):
            raise AttributeError(item)
        ds = DATA_NAME_TO_DATASTORE_TYPE.get(item)
        if ds is None:
            raise exceptions.UnknownData(f"Couldn't find any data named '{item}' on {self.sim}.")
        raise exceptions.MissingDatastore(
            f"Couldn't get data '{item}' for {self.sim} because it does not include a {ds.__name__} datastore."
        )


DATA_NAME_TO_DATASTORE_TYPE = {}


class Datastore:
    # True: ``store`` runs at every data time (the run loop stops there)
    stores_at_data_times = False

    def init(self, sim):
        self.sim = sim
        self.spec = sim.spec
        self.attach()

    def store(self):  # host-side datastores fill at data times
        pass

    def attach(self):
        raise NotImplementedError

    def pull(self, norm, ips):
        """Receive the device reductions (norm[n_data], ips[n_states, n_data])."""

    def __repr__(self):
        return self.__class__.__name__


def link_property_to_data(datastore_type, method):
    def get(data):
        try:
            return getattr(data.sim.datastores_by_type[datastore_type], method.__name__)()
        except KeyError:
            raise exceptions.MissingDatastore(
                f"Couldn't get data {method.__name__} for {data.sim} because it does not include a "
                f"{datastore_type.__name__} datastore."
            )

    return property(get)


class Fields(Datastore):
    """E(t) and A(t) at the data times (data.py:152-181).  The reference
    integrates E over times_to_current by Simpson's rule at every data time
    (pulses.py:58-77), O(n) each and O(n^2) per run when data are stored every
    step; here every prefix integral of the run comes from one O(n) pass with
    the same formulas (``potentials.vector_potential_table``), made once per
    run and indexed at the data times."""

    def init(self, sim):
        self.electric_field_amplitude = sim.get_blank_data()
        self.vector_potential_amplitude = sim.get_blank_data()
        self._a_table = None
        super().init(sim)

    def attach(self):
        self.sim.data.electric_field_amplitude = self.electric_field_amplitude
        self.sim.data.vector_potential_amplitude = self.vector_potential_amplitude

    def _vector_potential(self, t_index):
        if self._a_table is None:
            self._a_table = potentials.vector_potential_table(self.spec.electric_potential, self.sim.times)
        return self._a_table[t_index]

    def pull(self, norm, ips):
        sim = self.sim
        ep = self.spec.electric_potential
        for k, t_index in enumerate(sim.data_indices):
            if t_index > sim.time_index or not np.isnan(self.electric_field_amplitude[k]) and k > 0:
                continue
            self.electric_field_amplitude[k] = ep.get_electric_field_amplitude(sim.times[t_index])
            self.vector_potential_amplitude[k] = self._vector_potential(t_index)


DATA_NAME_TO_DATASTORE_TYPE.update({"electric_field_amplitude": Fields, "vector_potential_amplitude": Fields})


class Norm(Datastore):
    def init(self, sim):
        self.norm = sim.get_blank_data()
        super().init(sim)

    def attach(self):
        self.sim.data.norm = self.norm

    def pull(self, norm, ips):
        # slots the device has not written (NaN) keep their host value, which
        # matters after a reload from a checkpoint
        self.norm[:] = np.where(np.isnan(norm), self.norm, norm)


DATA_NAME_TO_DATASTORE_TYPE.update({"norm": Norm})


class InnerProducts(Datastore):
    def init(self, sim):
        self.inner_products = {state: sim.get_blank_data(dtype=np.complex128) for state in sim.spec.test_states}
        super().init(sim)

    def attach(self):
        self.sim.data.inner_products = self.inner_products
        self.sim.data.initial_state_inner_product = self.inner_products[self.spec.initial_state]

    def pull(self, norm, ips):
        for k, state in enumerate(self.spec.test_states):
            cur = self.inner_products[state]
            cur[:] = np.where(np.isnan(ips[k]), cur, ips[k])

    def state_overlaps(self):
        return {state: np.abs(ip) ** 2 for state, ip in self.inner_products.items()}

    def initial_state_overlap(self):
        return np.abs(self.inner_products[self.spec.initial_state]) ** 2

    def bound_state_overlap(self):
        return sum(o for s, o in self.state_overlaps().items() if s.bound)

    def free_state_overlap(self):
        return sum(o for s, o in self.state_overlaps().items() if s.free)

    def total_state_overlap(self):
        return sum(self.state_overlaps().values())


Data.state_overlaps = link_property_to_data(InnerProducts, InnerProducts.state_overlaps)
Data.initial_state_overlap = link_property_to_data(InnerProducts, InnerProducts.initial_state_overlap)
Data.bound_state_overlap = link_property_to_data(InnerProducts, InnerProducts.bound_state_overlap)
Data.free_state_overlap = link_property_to_data(InnerProducts, InnerProducts.free_state_overlap)
Data.total_state_overlap = link_property_to_data(InnerProducts, InnerProducts.total_state_overlap)

DATA_NAME_TO_DATASTORE_TYPE.update(
    {
        "inner_products": InnerProducts,
        "initial_state_inner_product": InnerProducts,
        "state_overlaps": InnerProducts,
        "initial_state_overlap": InnerProducts,
        "bound_state_overlap": InnerProducts,
        "free_state_overlap": InnerProducts,
        "total_state_overlap": InnerProducts,
    }
)

class ZExpectationValue(Datastore):
    """<z> at the data times (data.py:344-375): on the device, the F-order
    dipole operator on a spherical-harmonic mesh, z |g|^2 on line and
    cylindrical meshes."""

    stores_at_data_times = True

    def init(self, sim):
        self.z_expectation_value = sim.get_blank_data()
        super().init(sim)

    def store(self):
        self.z_expectation_value[self.sim.data_time_index] = self.sim.mesh.z_expectation_value()

    def attach(self):
        self.sim.data.z_expectation_value = self.z_expectation_value

    def z_dipole_moment_expectation_value(self):
        return self.spec.test_charge * self.z_expectation_value


Data.z_dipole_moment_expectation_value = link_property_to_data(
    ZExpectationValue, ZExpectationValue.z_dipole_moment_expectation_value)
DATA_NAME_TO_DATASTORE_TYPE.update({"z_expectation_value": ZExpectationValue,
                                    "z_dipole_moment_expectation_value": ZExpectationValue})


class RExpectationValue(Datastore):
    """<r> at the data times (data.py:378-395)."""

    stores_at_data_times = True

    def init(self, sim):
        self.r_expectation_value = sim.get_blank_data()
        super().init(sim)

    def store(self):
        self.r_expectation_value[self.sim.data_time_index] = self.sim.mesh.r_expectation_value()

    def attach(self):
        self.sim.data.r_expectation_value = self.r_expectation_value


DATA_NAME_TO_DATASTORE_TYPE.update({"r_expectation_value": RExpectationValue})


class NormWithinRadius(Datastore):
    """The norm of the part of the mesh with r <= R for each R (data.py:398-429;
    on a line r is the signed z coordinate, as the reference's r_mesh)."""

    stores_at_data_times = True

    def __init__(self, radii=()):
        self.radii = tuple(sorted(radii))

    def init(self, sim):
        self.norm_within_radius = {r: sim.get_blank_data() for r in self.radii}
        super().init(sim)

    def store(self):
        vals = self.sim.mesh.norm_within_radius(self.radii)
        for r, v in zip(self.radii, vals):
            self.norm_within_radius[r][self.sim.data_time_index] = v

    def attach(self):
        self.sim.data.norm_within_radius = self.norm_within_radius


DATA_NAME_TO_DATASTORE_TYPE.update({"norm_within_radius": NormWithinRadius})


class NormBySphericalHarmonic(Datastore):
    """The norm in each spherical harmonic (data.py:432-454), keyed like the
    specification's ``spherical_harmonics``."""

    stores_at_data_times = True

    def init(self, sim):
        self.norm_by_l = {sph: sim.get_blank_data() for sph in sim.spec.spherical_harmonics}
        super().init(sim)

    def store(self):
        for sph, v in zip(self.spec.spherical_harmonics, self.sim.mesh.norm_by_l()):
            self.norm_by_l[sph][self.sim.data_time_index] = v

    def attach(self):
        self.sim.data.norm_by_sph_harm = self.norm_by_l


DATA_NAME_TO_DATASTORE_TYPE.update({"norm_by_l": NormBySphericalHarmonic})

class InternalEnergyExpectationValue(Datastore):
    """<H0> at the data times (data.py:290-313): a device reduction of the
    internal Hamiltonian's expectation value."""

    stores_at_data_times = True

    def init(self, sim):
        self.internal_energy_expectation_value = sim.get_blank_data()
        super().init(sim)

    def store(self):
        self.internal_energy_expectation_value[self.sim.data_time_index] = (
            self.sim.mesh.internal_energy_expectation_value())

    def attach(self):
        self.sim.data.internal_energy_expectation_value = self.internal_energy_expectation_value


DATA_NAME_TO_DATASTORE_TYPE.update({"internal_energy_expectation_value": InternalEnergyExpectationValue})


class TotalEnergyExpectationValue(Datastore):
    """<H0 + V(t)> at the data times (data.py:316-340): the internal
    Hamiltonian plus the interaction at the data time."""

    stores_at_data_times = True

    def init(self, sim):
        self.total_energy_expectation_value = sim.get_blank_data()
        super().init(sim)

    def store(self):
        self.total_energy_expectation_value[self.sim.data_time_index] = (
            self.sim.mesh.total_energy_expectation_value())

    def attach(self):
        self.sim.data.total_energy_expectation_value = self.total_energy_expectation_value


DATA_NAME_TO_DATASTORE_TYPE.update({"total_energy_expectation_value": TotalEnergyExpectationValue})


class DirectionalRadialProbabilityCurrent(Datastore):
    """The radial probability current through each shell r_j at the data
    times, for z > 0 and z < 0 (data.py:467-530), on spherical-harmonic
    meshes (SphericalHarmonicMesh.radial_probability_current).  Arrays of
    shape (data times, r_points), NaN until stored.  The reference's own
    class reads ``self.sim`` in ``init`` before the base class sets it, and
    its mesh method calls the current operator without the mesh, so it does
    not run there; this one computes what those lines describe."""

    stores_at_data_times = True

    def init(self, sim):
        if not hasattr(sim.mesh, "radial_probability_current"):
            raise exceptions.UnsupportedMesh(
                f"DirectionalRadialProbabilityCurrent needs a spherical-harmonic mesh, not {type(sim.mesh).__name__}")
        shape = (sim.data_time_steps, sim.spec.r_points)
        self.radial_probability_current__pos_z = np.full(shape, np.nan)
        self.radial_probability_current__neg_z = np.full(shape, np.nan)
        super().init(sim)

    def store(self):
        pos, neg = self.sim.mesh.radial_probability_current()
        self.radial_probability_current__pos_z[self.sim.data_time_index] = pos
        self.radial_probability_current__neg_z[self.sim.data_time_index] = neg

    def attach(self):
        self.sim.data.radial_probability_current__pos_z = self.radial_probability_current__pos_z
        self.sim.data.radial_probability_current__neg_z = self.radial_probability_current__neg_z

    def radial_probability_current__total(self):
        return self.radial_probability_current__pos_z + self.radial_probability_current__neg_z


Data.radial_probability_current__total = link_property_to_data(
    DirectionalRadialProbabilityCurrent, DirectionalRadialProbabilityCurrent.radial_probability_current__total)
DATA_NAME_TO_DATASTORE_TYPE.update({
    "radial_probability_current__pos_z": DirectionalRadialProbabilityCurrent,
    "radial_probability_current__neg_z": DirectionalRadialProbabilityCurrent,
    "radial_probability_current__total": DirectionalRadialProbabilityCurrent,
})

DEFAULT_DATASTORE_TYPES = (Fields, Norm, InnerProducts)
