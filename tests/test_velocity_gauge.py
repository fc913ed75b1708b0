"""Velocity-gauge host side: the vector-potential table, the operator tables
and the combinations the device path rejects.  The device runs are checked
against the reference's velocity-gauge fixtures in test_gpu_parity.py."""

import numpy as np
import pytest
from scipy import integrate

from ionization_gb300 import exceptions, potentials
from oracle import mesh as om

from .conftest import load_golden
from .specs import product_spec


@pytest.mark.parametrize("n", [2, 3, 4, 5, 6, 101, 1000])
def test_prefix_simpson_matches_scipy_at_every_step(n):
    """A(times[k]) for every k from one pass equals scipy's Simpson integral
    of each prefix (what the reference evaluates at every step)."""
    rng = np.random.default_rng(n)
    t = np.cumsum(rng.uniform(0.5, 1.5, n)) * 0.02  # irregular spacing as well
    y = np.sin(3 * t) * np.exp(-t)
    got = potentials.simpson_prefix_integrals(y, t)
    want = np.array([0.0] + [integrate.simpson(y=y[: k + 1], x=t[: k + 1]) for k in range(1, n)])
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-15 * max(1.0, np.max(np.abs(want))))


def _host_tables(kind, name, **kw):
    params, _ = load_golden(name)
    spec = product_spec(kind, params, **kw)
    spec.host_only = True
    return params, spec.to_sim().mesh.tables


def test_sh_velocity_tables_match_the_oracle():
    params, tab = _host_tables("sh", "sh_velocity_small_oddNr_oddL")
    st = om.build_from_params("sh", params)
    times = om.get_times(params["time_initial"], params["time_final"], params["time_step"])
    assert tab.gauge == 1
    # h1: rq_j c_l (l+1) on the F-order neighbours (l, l+1) of row j
    h1 = (tab.rq[None, :] * (tab.cl * (np.arange(tab.n_l) + 1))[:, None])[:-1].T.ravel()
    want = np.append(st.h1_off, 0.0).reshape(tab.n_r, tab.n_l)[:, :-1].ravel()  # F order: k = j L + l
    np.testing.assert_allclose(h1, want, rtol=1e-14, atol=0)
    np.testing.assert_allclose(tab.h2r, st.h2_r, rtol=1e-14, atol=0)
    A = [om.vector_potential(st.pulse, times[: k + 1]) for k in range(1, len(times))]
    np.testing.assert_allclose(tab.efield[1:], A, rtol=0, atol=1e-15)


def test_line_velocity_tables():
    params, tab = _host_tables("line", "line_velocity_small")
    z = np.linspace(-params["z_bound"], params["z_bound"], params["z_points"])
    assert tab.gauge == 1
    assert tab.vcoef == pytest.approx(-1.0 / (params["test_mass"] * 2 * (z[1] - z[0])), rel=1e-14)


@pytest.mark.parametrize("method,precision", [("AlternatingDirectionImplicit", "c128"), ("SplitInteractionOperator", "c64x")])
def test_line_velocity_unsupported_forms_raise(method, precision):
    params, _ = load_golden("line_velocity_small")
    params = dict(params, method=method)
    spec = product_spec("line", params, precision=precision)
    spec.host_only = True
    with pytest.raises(exceptions.UnsupportedMesh):
        spec.to_sim()
