"""Position expectation values and partial norms: the ZExpectationValue,
RExpectationValue, NormWithinRadius and NormBySphericalHarmonic datastores.

The fixtures come from the reference run with those datastores
(tests/golden/make_golden.py --only obs).  The reference cannot run two of
them as written: a line's <z> raises (LineLengthGaugeOperators.z returns a
tuple), and NormBySphericalHarmonic.init reads ``spec`` before it is set.  So
the line fixture holds NormWithinRadius only, and the SH fixture holds the
reference's ``norm_by_l()`` at the final time.  The oracle is checked against
the fixtures first; the device reductions are then checked against both."""

import numpy as np
import pytest

from oracle import mesh as om

from .conftest import load_golden
from .specs import product_spec

TOL = 1e-10


def _oracle(kind, name):
    params, z = load_golden(name)
    radii = [float(r) for r in z["radii"]]
    out = om.run_from_params(kind, params, radii=radii)
    return params, z, radii, out


@pytest.mark.parametrize("kind,name", [("line", "line_observables_small"), ("sh", "sh_observables_small"),
                                       ("cyl", "cyl_observables_small")])
def test_oracle_observables_match_reference(kind, name):
    params, z, radii, out = _oracle(kind, name)
    obs = out["observed"]
    within = np.array([o["within"] for o in obs]).T
    np.testing.assert_allclose(within, z["norm_within_radius"], rtol=0, atol=1e-12)
    if kind != "line":
        np.testing.assert_allclose([o["z"] for o in obs], z["z_expectation_value"], rtol=0, atol=1e-12)
        np.testing.assert_allclose([o["r"] for o in obs], z["r_expectation_value"], rtol=0, atol=1e-12)
    if kind == "sh":
        np.testing.assert_allclose(obs[-1]["by_l"], z["norm_by_l_final"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("kind,name", [("line", "line_observables_small"), ("sh", "sh_observables_small"),
                                       ("cyl", "cyl_observables_small")])
def test_fields_tables_match_reference(kind, name):
    """The Fields datastore's host tables: E at the data times and A from the
    one-pass prefix integrals, against the reference's per-data-time Simpson
    integrals (data.py:152-181)."""
    from ionization_gb300 import potentials

    from .specs import pulse

    params, z = load_golden(name)
    times = z["times"]
    idx = np.searchsorted(times, z["data_times"])
    ep = pulse(params["pulse"])
    a = potentials.vector_potential_table(ep, times)[idx]
    e = np.array([ep.get_electric_field_amplitude(t) for t in times[idx]])
    np.testing.assert_array_equal(e, z["electric_field_amplitude"])
    np.testing.assert_allclose(a, z["vector_potential_amplitude"], rtol=0, atol=1e-15)


def _product_datastores(kind, radii):
    from ionization_gb300.mesh import data

    stores = [data.Fields(), data.Norm(), data.InnerProducts(), data.NormWithinRadius(radii=radii),
              data.ZExpectationValue(), data.RExpectationValue()]
    if kind == "sh":
        stores.append(data.NormBySphericalHarmonic())
    return stores


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", [("line", "line_observables_small"), ("sh", "sh_observables_small"),
                                       ("cyl", "cyl_observables_small")])
def test_device_observables_c128(cuda, kind, name):
    params, z, radii, out = _oracle(kind, name)
    sim = product_spec(kind, params, datastores=_product_datastores(kind, radii)).to_sim()
    sim.run()
    within = np.array([sim.data.norm_within_radius[r] for r in sorted(radii)])
    np.testing.assert_allclose(within, z["norm_within_radius"], rtol=0, atol=TOL)
    np.testing.assert_array_equal(sim.data.electric_field_amplitude, z["electric_field_amplitude"])
    np.testing.assert_allclose(sim.data.vector_potential_amplitude, z["vector_potential_amplitude"], rtol=0,
                               atol=1e-15)
    obs = out["observed"]
    np.testing.assert_allclose(sim.data.z_expectation_value, [o["z"] for o in obs], rtol=0, atol=TOL)
    np.testing.assert_allclose(sim.data.r_expectation_value, [o["r"] for o in obs], rtol=0, atol=TOL)
    if kind != "line":
        np.testing.assert_allclose(sim.data.z_expectation_value, z["z_expectation_value"], rtol=0, atol=TOL)
        np.testing.assert_allclose(sim.data.r_expectation_value, z["r_expectation_value"], rtol=0, atol=TOL)
    if kind == "sh":
        by_l = np.array([sim.data.norm_by_sph_harm[h][-1] for h in sim.spec.spherical_harmonics])
        np.testing.assert_allclose(by_l, z["norm_by_l_final"], rtol=0, atol=TOL)
        np.testing.assert_allclose(sum(sim.data.norm_by_sph_harm.values()), sim.data.norm, rtol=0, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["c64", "c64x"])
def test_device_observables_sh_complex64(cuda, precision):
    params, z, radii, out = _oracle("sh", "sh_observables_small")
    sim = product_spec("sh", params, precision=precision, datastores=_product_datastores("sh", radii)).to_sim()
    sim.run()
    np.testing.assert_allclose(sim.data.z_expectation_value, z["z_expectation_value"], rtol=0, atol=1e-5)
    np.testing.assert_allclose(sim.data.r_expectation_value, z["r_expectation_value"], rtol=0, atol=1e-4)
    within = np.array([sim.data.norm_within_radius[r] for r in sorted(radii)])
    np.testing.assert_allclose(within, z["norm_within_radius"], rtol=0, atol=1e-5)
