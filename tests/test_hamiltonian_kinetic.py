"""kinetic_energy_derivation="hamiltonian" on the spherical-harmonic mesh
(SphericalHarmonicLengthGaugeOperators.kinetic_energy_from_hamiltonian,
mesh_operators.py:863-887): the radial kinetic energy of the flattened
(l, r) mesh, whose couplings also join the last r of each l to the first r of
the next.  The device solves each line and adds that coupling through
precomputed spikes; the fixture is a reference run
(tests/golden/make_golden.py --only ham) on a short grid that the pulse
drives to its edge, so the coupling acts."""

import numpy as np
import pytest

from .conftest import load_golden, rel_l2
from .specs import product_spec


def test_host_tables_couple_consecutive_lines():
    params, _ = load_golden("sh_hamiltonian_small")
    sim = product_spec("sh", params, host_only=True).to_sim()
    tb = sim.mesh.operators.device_tables(sim.mesh)
    assert tb["cross"] is not None and tb["cross"] == tb["hoff"][0]
    h = sim.mesh.operators.internal_hamiltonian(sim.mesh).operators[0].matrix
    nr = params["r_points"]
    assert h.diagonal(1)[nr - 1] == tb["cross"]  # (l=0, last r) - (l=1, first r)
    np.testing.assert_array_equal(sim.mesh.tables.hd, tb["hd"])


@pytest.mark.parametrize("precision", ["c64", "c64x"])
def test_complex64_forms_are_refused(precision):
    from ionization_gb300 import exceptions

    params, _ = load_golden("sh_hamiltonian_small")
    with pytest.raises(exceptions.UnsupportedMesh, match="hamiltonian"):
        product_spec("sh", params, precision=precision, host_only=True).to_sim()


def test_numeric_eigenstates_raise_like_the_reference():
    params, _ = load_golden("sh_hamiltonian_small")
    with pytest.raises(NotImplementedError):
        product_spec("sh", params, use_numeric_eigenstates=True, host_only=True).to_sim()


@pytest.mark.gpu
def test_hamiltonian_kinetic_matches_reference(cuda):
    from ionization_gb300 import mesh

    params, z = load_golden("sh_hamiltonian_small")
    sim = product_spec("sh", params, datastores=[mesh.Fields(), mesh.Norm(), mesh.InnerProducts(),
                                                 mesh.InternalEnergyExpectationValue(),
                                                 mesh.TotalEnergyExpectationValue()]).to_sim()
    sim.run()
    assert rel_l2(sim.mesh.g, z["g_final"]) < 1e-10
    np.testing.assert_allclose(sim.data.norm, z["norm"], rtol=0, atol=1e-10)
    ips = np.array([sim.data.inner_products[s] for s in sim.spec.test_states])
    np.testing.assert_allclose(ips, z["inner_products"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(sim.data.internal_energy_expectation_value, z["internal_energy_expectation_value"],
                               rtol=0, atol=1e-10)
    np.testing.assert_allclose(sim.data.total_energy_expectation_value, z["total_energy_expectation_value"],
                               rtol=0, atol=1e-10)


@pytest.mark.gpu
def test_the_line_coupling_matters(cuda):
    """Without the fix-up (the plan flag cleared) the same run misses the
    reference by far more than the parity bound."""
    from ionization_gb300 import _native as nat

    params, z = load_golden("sh_hamiltonian_small")
    sim = product_spec("sh", params).to_sim()
    plan = sim.mesh._batch.plan
    plan.flags &= ~nat.ION_SH_COUPLED
    sim.run()
    assert rel_l2(sim.mesh.g, z["g_final"]) > 1e-6
