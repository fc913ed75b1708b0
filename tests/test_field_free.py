"""Field-free evolution keeps an eigenstate an eigenstate: with no electric
potential, a run from a numeric hydrogen eigenstate ends with the norm and
every test-state overlap it started with, to 1e-14, for the length gauge
under ADI and under the split operator and for the velocity gauge under the
split operator.  Mirrors the reference's own test of the same name
(tests/mesh/test_sims.py:29-82, states n < 3)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATES = [(n, l) for n in range(3) for l in range(n)]
FORMS = [("length", "adi"), ("length", "split"), ("velocity", "split")]


@pytest.mark.parametrize("form", FORMS, ids=lambda f: f"{f[0]}-{f[1]}")
@pytest.mark.parametrize("nl", STATES, ids=lambda s: f"n{s[0]}l{s[1]}")
def test_with_no_potential_final_state_is_initial_state(cuda, nl, form):
    import ionization_gb300 as ion
    from ionization_gb300 import units as u

    operators = (ion.mesh.SphericalHarmonicLengthGaugeOperators() if form[0] == "length"
                 else ion.mesh.SphericalHarmonicVelocityGaugeOperators())
    method = ion.mesh.AlternatingDirectionImplicit() if form[1] == "adi" else ion.mesh.SplitInteractionOperator()
    sim = ion.mesh.SphericalHarmonicSpecification(
        "field_free",
        initial_state=ion.states.HydrogenBoundState(*nl),
        operators=operators,
        evolution_method=method,
        time_initial=0,
        time_final=100 * u.asec,
        time_step=1 * u.asec,
        r_bound=50 * u.bohr_radius,
        r_points=250,
        l_bound=30,
        use_numeric_eigenstates=True,
        numeric_eigenstate_max_energy=10 * u.eV,
        numeric_eigenstate_max_angular_momentum=10,
    ).to_sim()
    sim.run()
    overlaps = sim.data.state_overlaps
    first = np.array([o[0] for o in overlaps.values()])
    last = np.array([o[-1] for o in overlaps.values()])
    assert np.allclose(sim.data.norm[0], sim.data.norm[-1], atol=1e-14)
    assert np.allclose(first, last, atol=1e-14)
