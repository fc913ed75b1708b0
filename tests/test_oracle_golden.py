"""The oracle (CPU restatement) against fixtures produced by the reference.

These pin the oracle: every case here was generated by running the reference
ionization library itself (tests/golden/make_golden.py)."""

import numpy as np
import pytest

import oracle
from oracle import mesh as om

from .conftest import load_golden, rel_l2


def test_tdma_matches_cy_tdma_bitwise():
    _, z = load_golden("tdma")
    for i in range(9):
        x = oracle.tdma_from_dia(z[f"n{i}_data"], z[f"n{i}_d"])
        np.testing.assert_array_equal(x, z[f"n{i}_x"])
    x = oracle.tdma_from_dia(z["batch_data"], z["batch_d"])
    np.testing.assert_array_equal(x, z["batch_x"])


def test_tdma_batched_equals_single_call():
    _, z = load_golden("tdma")
    nl, n = z["batch_shape"]
    data = z["batch_data"]
    sub = data[0][:-1].copy()
    sup = data[2][1:].copy()
    keep = np.ones(nl * n - 1, bool)
    keep[n - 1 :: n] = False
    x = oracle.tdma_batched(
        sub[keep].reshape(nl, n - 1), data[1].reshape(nl, n), sup[keep].reshape(nl, n - 1), z["batch_d"].reshape(nl, n)
    )
    np.testing.assert_array_equal(x.ravel(), z["batch_x"])


CASES = [
    ("line", "line_adi_small"),
    ("line", "line_split_small"),
    ("sh", "sh_split_small_evenL"),
    ("sh", "sh_split_small_oddL"),
    ("sh", "sh_split_small_oddNr_oddL"),
    ("cyl", "cyl_adi_small"),
    # velocity gauge (SphericalHarmonicVelocityGaugeOperators, LineVelocityGaugeOperators)
    ("sh", "sh_velocity_small_evenL"),
    ("sh", "sh_velocity_small_oddNr_oddL"),
    ("sh", "sh_velocity_small_evenNr_oddL"),
    ("line", "line_velocity_small"),
    ("line", "line_velocity_small_odd"),
    # SphericalHarmonicMesh with AlternatingDirectionImplicit
    ("sh", "sh_adi_small_evenL"),
    ("sh", "sh_adi_small_oddNr_oddL"),
    # RectangleMesh with AlternatingDirectionImplicit
    ("rect", "rect_adi_small"),
    ("rect", "rect_adi_small_odd"),
    # SphericalSliceMesh with AlternatingDirectionImplicit
    ("slice", "slice_adi_small"),
    ("slice", "slice_adi_small_odd"),
]


@pytest.mark.parametrize("kind,name", CASES)
def test_oracle_run_matches_reference(kind, name):
    params, z = load_golden(name)
    out = om.run_from_params(kind, params)
    np.testing.assert_array_equal(out["times"], z["times"])
    assert rel_l2(out["g_initial"], z["g_initial"]) < 1e-14  # fixtures come from x86 libm
    assert rel_l2(out["g_final"], z["g_final"]) < 1e-13
    np.testing.assert_allclose(out["norm"], z["norm"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(out["inner_products"], z["inner_products"], rtol=0, atol=1e-13)


def test_oracle_full_line_matches_reference():
    params, z = load_golden("line_cfg1_full")
    out = om.run_from_params("line", params)
    assert rel_l2(out["g_final"], z["g_final"]) < 1e-12
    np.testing.assert_allclose(out["norm"], z["norm"], rtol=0, atol=1e-12)


def test_pulse_mapping_is_sin2_envelope():
    """E0 sin^2(pi t/T) cos(w t + cep) equals CosSquaredPulse centred at T/2
    with phase cep + N pi."""
    from ionization_gb300.potentials import CosSquaredPulse

    E0, w, N, cep = 0.05, 0.057, 4, 0.3
    p = CosSquaredPulse.from_sin2_envelope(E0, w, N, cep)
    T = N * 2 * np.pi / w
    t = np.linspace(0, T, 1001)
    want = E0 * np.sin(np.pi * t / T) ** 2 * np.cos(w * t + cep)
    np.testing.assert_allclose(p.get_electric_field_amplitude(t), want, atol=1e-12)
