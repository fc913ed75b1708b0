"""The numeric eigenstate basis (use_numeric_eigenstates=True): the device's
batched tridiagonal eigensolver (Sturm bisection + inverse iteration) and the
spherical-harmonic run that uses the basis as its test and initial states.

The reference finds the basis with scipy's eigsh on complex-typed matrices,
so its eigenvectors carry an arbitrary complex phase each; comparisons are
of energies, of |<numeric state | psi>| and of psi up to the initial
(ground) state's phase."""

import numpy as np
import pytest

from oracle import mesh as om

from .conftest import load_golden, rel_l2
from .specs import product_spec


def _fixture_basis():
    params, z = load_golden("sh_numeric_small")
    return params, z


def test_oracle_basis_matches_the_reference():
    """LAPACK's tridiagonal eigenpairs restate the reference's eigsh basis."""
    params, z = _fixture_basis()
    basis = om.numeric_eigenbasis(params["r_points"], params["r_bound"], params["numeric_eigenstate_max_energy"],
                                  params["numeric_eigenstate_max_angular_momentum"])
    assert len(basis) == len(z["numeric_energy"])
    np.testing.assert_allclose([b[1] for b in basis], z["numeric_energy"], rtol=0, atol=1e-11)
    assert [b[0] for b in basis] == list(z["numeric_l"])
    dr = params["r_bound"] / (params["r_points"] - 1)
    for (l, _, v), g in zip(basis, z["numeric_g"]):
        overlap = abs(np.sum(np.conj(g) * v) * dr)  # both normalised on the mesh
        assert overlap == pytest.approx(1.0, abs=1e-9)


@pytest.mark.gpu
def test_device_eigenpairs_match_lapack(cuda):
    from scipy.linalg import eigh_tridiagonal

    from ionization_gb300 import _device as dev

    rng = np.random.default_rng(7)
    n = 200
    d = rng.normal(size=(3, n)) * np.array([[1.0], [10.0], [0.1]])
    e = rng.normal(size=(3, n - 1))
    cap = 0.5
    got = dev.tridiagonal_eigenpairs(d, e, cap, n - 2)
    for m in range(3):
        w, v = eigh_tridiagonal(d[m], e[m], select="v", select_range=(-np.inf, cap))
        gw, gv = got[m]
        assert len(gw) == len(w)
        np.testing.assert_allclose(gw, w, rtol=0, atol=1e-12 * np.max(np.abs(d[m]) + 2))
        ov = np.abs(np.sum(gv * v.T, axis=1))
        assert np.min(ov) > 1 - 1e-9
        np.testing.assert_allclose(gv @ gv.T, np.eye(len(gw)), rtol=0, atol=1e-9)


@pytest.mark.gpu
def test_numeric_basis_run_matches_the_reference(cuda):
    from ionization_gb300 import mesh, states

    params, z = _fixture_basis()
    spec = product_spec("sh", params, use_numeric_eigenstates=True,
                        numeric_eigenstate_max_energy=params["numeric_eigenstate_max_energy"],
                        numeric_eigenstate_max_angular_momentum=params["numeric_eigenstate_max_angular_momentum"],
                        evolution_method=mesh.SplitInteractionOperator())
    sim = spec.to_sim()
    ts = list(sim.spec.test_states)
    assert all(isinstance(s, states.NumericSphericalHarmonicState) for s in ts)
    assert isinstance(sim.spec.initial_state, states.NumericSphericalHarmonicState)
    np.testing.assert_allclose([s.energy for s in ts], z["numeric_energy"], rtol=0, atol=1e-11)
    assert [s.l for s in ts] == list(z["numeric_l"])
    assert [s.bound for s in ts] == list(z["numeric_bound"])
    # the radial vectors, up to each state's phase
    for s, g in zip(ts, z["numeric_g"]):
        mine = sim.mesh.get_radial_g_for_state(s)
        ph = np.vdot(mine, g)
        assert abs(ph) * params["r_bound"] / (params["r_points"] - 1) == pytest.approx(1.0, abs=1e-9)
    sim.run()
    np.testing.assert_allclose(sim.data.norm, z["norm"], rtol=0, atol=1e-10)
    ips = np.array([sim.data.inner_products[s] for s in ts])
    np.testing.assert_allclose(np.abs(ips), np.abs(z["inner_products"]), rtol=0, atol=1e-10)
    # psi up to the initial state's phase
    g0 = sim.mesh.get_g_for_state(sim.spec.initial_state)
    phase = np.vdot(g0.ravel(), z["g_initial"].ravel())
    phase /= abs(phase)
    assert rel_l2(np.asarray(sim.mesh.g) * phase, z["g_final"]) < 1e-9
