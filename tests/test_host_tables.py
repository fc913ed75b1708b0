"""Host-side coefficient build of the product against the oracle (CPU only).

The device kernels consume FP64 tables built on the host; these must be
identical to the reference's operator diagonals (the oracle restates them and
is itself pinned to the reference by test_oracle_golden)."""

import numpy as np
import pytest

from oracle import mesh as om

from .conftest import load_golden
from .specs import product_spec


@pytest.mark.parametrize("name", ["line_adi_small", "line_split_small"])
def test_line_tables(name):
    params, z = load_golden(name)
    sim = product_spec("line", params, host_only=True).to_sim()
    tb = sim.mesh.tables
    ref = om.build_from_params("line", params)
    np.testing.assert_array_equal(tb.hd, ref.H0.diag.real)
    np.testing.assert_array_equal(tb.hoff, ref.H0.sub.real)
    np.testing.assert_array_equal(tb.mask, ref.mask)
    np.testing.assert_allclose(tb.g0, z["g_initial"], rtol=1e-14, atol=1e-300)
    times = om.get_times(params["time_initial"], params["time_final"], params["time_step"])
    np.testing.assert_array_equal(sim.times, times)
    np.testing.assert_array_equal(tb.efield[1:], ref.pulse.field(times[1:]))
    np.testing.assert_array_equal(tb.zq * 0.3, (-ref.z * -1.0) * 0.3)


@pytest.mark.parametrize("name", ["sh_split_small_evenL", "sh_split_small_oddL", "sh_split_small_oddNr_oddL"])
def test_sh_tables(name):
    params, z = load_golden(name)
    sim = product_spec("sh", params, host_only=True).to_sim()
    tb = sim.mesh.tables
    ref = om.build_from_params("sh", params)
    np.testing.assert_array_equal(tb.hd, ref.H0.diag.real)
    nr, L = params["r_points"], params["l_bound"]
    np.testing.assert_array_equal(tb.hoff, ref.H0.sub.real[: nr - 1])
    # the rotation coupling c_l * r evaluated on the fly equals the reference's table
    k = np.arange(nr * L - 1)
    coupling = np.where((k + 1) % L != 0, tb.cl[k % L] * tb.rq[k // L], 0)
    np.testing.assert_array_equal(coupling, ref.l_off.real)
    np.testing.assert_array_equal(tb.mask, ref.mask[0])
    np.testing.assert_allclose(tb.g0, z["g_initial"], rtol=1e-14, atol=1e-300)
    times = sim.times
    np.testing.assert_array_equal(tb.efield[1:], ref.pulse.field(times[1:] + params["time_step"] / 2))
    # test states: sorted like the reference, radial g identical
    for (n, l), sl, sg in zip(params["test_states"], tb.state_l, tb.state_g):
        assert sl == l
        np.testing.assert_array_equal(sg, ref.radial_g[(n, l)])
    # complex64 pieces reproduce the FP64 diagonal to rounding
    for l in (0, 1, L - 1):
        h = tb.kinv + l * (l + 1) * tb.cent
        if l == 0:
            h = h.copy()
            h[0] += tb.corr0
        np.testing.assert_allclose(h, tb.hd[l * nr:(l + 1) * nr], rtol=1e-13, atol=1e-10)


def test_cyl_tables():
    params, z = load_golden("cyl_adi_small")
    sim = product_spec("cyl", params, host_only=True).to_sim()
    tb = sim.mesh.tables
    ref = om.build_from_params("cyl", params)
    nz, nr = params["z_points"], params["rho_points"]
    np.testing.assert_array_equal(tb["hr_d"], ref.H_rho0.diag.real)
    np.testing.assert_array_equal(tb["hz_d"], np.reshape(ref.H_z0.diag.real, (nz, nr), "F").ravel())
    np.testing.assert_array_equal(tb["hr_off"], ref.H_rho0.sub.real[: nr - 1])
    np.testing.assert_array_equal(tb["hz_off"], ref.H_z0.sub.real[: nz - 1])
    np.testing.assert_allclose(tb["g0"], z["g_initial"], rtol=1e-14, atol=1e-300)
    for s, gs in zip(params["test_states"], tb["state_g"]):
        np.testing.assert_array_equal(gs.reshape(nz, nr), ref.test_g[tuple(s)])


def test_data_slots_match_reference_mask():
    from ionization_gb300 import _device as dev

    for tf in (0, 1, 7, 100, 101):
        for every in (-1, 1, 3, 10, 200):
            idx = np.arange(tf + 1)
            mask = om.data_mask(tf + 1, every)
            assert dev.n_data_slots(tf, every) == mask.sum()
            slots = np.cumsum(mask) - 1
            for t in idx:
                assert dev.is_data_time(t, tf, every) == bool(mask[t])
                if mask[t]:
                    assert dev.data_slot(t, tf, every) == slots[t]


def test_residual_packing_rounds_like_bf16():
    """The stored residual of a complex64 state (two bf16 in one word) is
    packed on the host with round-to-nearest-even, as the device packs it:
    torch's float32 -> bfloat16 conversion gives the same values, over
    magnitudes from subnormal to large, zeros and ties included."""
    import torch

    from ionization_gb300 import _device as dev

    rng = np.random.default_rng(1)
    n = 100_000
    x = (rng.normal(size=n) * np.exp(rng.uniform(-90, 5, n))
         + 1j * rng.normal(size=n) * np.exp(rng.uniform(-90, 5, n))).astype(np.complex64)
    x[:8] = 0
    x[8:16] = np.float32(1e-40) - 1j * np.float32(3e-42)
    x[16:18] = np.float32(1 + 2 ** -8) + 1j * np.float32(1 + 3 * 2 ** -8)  # ties: to even
    w = dev.lo_pack(x)
    assert w.dtype == np.int32 and w.shape == x.shape
    u = dev.lo_unpack(w)
    want_re = torch.from_numpy(x.real.copy()).to(torch.bfloat16).float().numpy()
    want_im = torch.from_numpy(x.imag.copy()).to(torch.bfloat16).float().numpy()
    assert np.array_equal(u.real.astype(np.float32), want_re)
    assert np.array_equal(u.imag.astype(np.float32), want_im)
    assert u[16] == 1 + 1j * (1 + 2 ** -6)


@pytest.mark.parametrize("kind,name", [("cyl", "cyl_adi_small"), ("rect", "rect_adi_small"),
                                       ("sh", "sh_adi_small_evenL")])
def test_adi_meshes_have_no_c64x_form(kind, name):
    """The two-direction ADI kernel pair has complex128 and complex64 forms;
    asking for the stored-residual form is refused before any device work."""
    from ionization_gb300 import exceptions

    params, _ = load_golden(name)
    with pytest.raises(exceptions.UnsupportedMesh, match="c64x"):
        product_spec(kind, params, precision="c64x", host_only=True).to_sim()


@pytest.mark.parametrize("precision", ["c64", "c64x"])
def test_spherical_slice_is_complex128_only(precision):
    from ionization_gb300 import exceptions

    params, _ = load_golden("slice_adi_small")
    with pytest.raises(exceptions.UnsupportedMesh, match="complex128"):
        product_spec("slice", params, precision=precision, host_only=True).to_sim()
