"""Energy expectation values and the radial probability current: the
InternalEnergyExpectationValue, TotalEnergyExpectationValue and
DirectionalRadialProbabilityCurrent datastores.

The fixtures come from the reference run with the energy datastores
(tests/golden/make_golden.py --only energy).  The reference cannot run its
DirectionalRadialProbabilityCurrent as written (its init reads ``sim`` before
it is set, and the mesh method calls the current operator without the
mesh); the fixture holds its store() at the final time with those two
arguments supplied.  CPU tests check the host-built operator tables and the
l-pair regrouping of the current against the fixtures with numpy; GPU tests
check the device reductions through the datastores."""

import numpy as np
import pytest

from .conftest import load_golden
from .specs import product_spec

TOL = 1e-10
CASES = [("line", "line_energy_small"), ("line", "line_energy_velocity_small"), ("sh", "sh_energy_small"),
         ("cyl", "cyl_energy_small"), ("rect", "rect_energy_small"), ("sh", "sh_hamiltonian_small")]


def _apply(ops, g):
    """weight-free <g|H|g> of (diag, off_b, off_a, flags) tables, in numpy."""
    from ionization_gb300 import _native as nat

    diag, off_b, off_a, flags = ops
    shape = g.shape
    out = 0.0
    if diag is not None:
        out += np.sum(np.broadcast_to(diag, shape) * np.abs(g) ** 2)
    if off_b is not None and flags & nat.ION_HOP_WRAP_B:  # the chain runs on over the flattened mesh
        c = np.broadcast_to(off_b, shape).reshape(-1)[:-1]
        z = np.conj(g.reshape(-1)[:-1]) * g.reshape(-1)[1:]
        out += np.sum(-2 * c * z.imag) if flags & nat.ION_HOP_IMAG_B else np.sum(2 * c * z.real)
        off_b = None
    for off, axis, imag in ((off_b, 1, flags & nat.ION_HOP_IMAG_B), (off_a, 0, flags & nat.ION_HOP_IMAG_A)):
        if off is None:
            continue
        c = np.broadcast_to(off, shape)
        x, y = (g[:, :-1], g[:, 1:]) if axis == 1 else (g[:-1, :], g[1:, :])
        cc = c[:, :-1] if axis == 1 else c[:-1, :]
        z = np.conj(x) * y
        out += np.sum(-2 * cc * z.imag) if imag else np.sum(2 * cc * z.real)
    return out


@pytest.mark.parametrize("kind,name", CASES)
def test_energy_tables_reproduce_reference(kind, name):
    """The host-built H0 and interaction tables, applied in numpy to the
    reference's final psi, give the reference's final internal and total
    energies (to rounding)."""
    params, z = load_golden(name)
    sim = product_spec(kind, params, host_only=True).to_sim()
    m = sim.mesh
    (na, nb), internal, inter, field = m._energy_operators()
    g = np.asarray(z["g_final"], dtype=np.complex128).reshape(na, nb)
    w = m.inner_product_multiplier
    e_int = w * _apply(internal, g)
    np.testing.assert_allclose(e_int, z["internal_energy_expectation_value"][-1], rtol=0, atol=1e-12)
    sim.time_index = len(sim.times) - 1  # sim.time follows it
    e_tot = e_int if inter is None else e_int + field() * w * _apply(inter, g)
    np.testing.assert_allclose(e_tot, z["total_energy_expectation_value"][-1], rtol=0, atol=1e-12)


def test_sph_harm_m0_matches_scipy():
    special = pytest.importorskip("scipy.special")
    if not hasattr(special, "sph_harm_y"):
        pytest.skip("scipy without sph_harm_y")
    from ionization_gb300.mesh.meshes import sph_harm_m0

    theta = np.linspace(0, np.pi, 181)
    ls = np.arange(60)
    want = np.array([special.sph_harm_y(l, 0, theta, 0.0).real for l in ls])
    np.testing.assert_allclose(sph_harm_m0(ls, theta), want, rtol=0, atol=1e-13)


def test_radial_current_regrouping_reproduces_reference():
    """The device form of the current, w = W u and Im(conj(w) . v) per shell
    with the hemisphere weights W built on the host, evaluated in numpy on
    the reference's final psi, gives the reference datastore's values."""
    from ionization_gb300 import units as u
    from ionization_gb300.mesh.meshes import sph_harm_m0

    params, z = load_golden("sh_energy_small")
    sim = product_spec("sh", params, host_only=True).to_sim()
    m = sim.mesh
    g = np.asarray(z["g_final"], dtype=np.complex128)
    L, nr = g.shape
    theta = np.linspace(0, np.pi, int(z["theta_points"]))
    y = sph_harm_m0(np.arange(L), theta)
    wt = u.twopi * np.abs(theta[1] - theta[0]) * np.sin(theta)
    up = theta <= np.pi / 2
    j = np.arange(1, nr, dtype=np.float64)
    od = (u.hbar / (2 * m.spec.test_mass * m.delta_r ** 3)) / (j ** 2 - 0.25)
    v = np.zeros_like(g)
    v[:, :-1] += od * g[:, 1:]
    v[:, 1:] -= od * g[:, :-1]
    for hemi, key in ((up, "radial_current_pos_z_final"), (~up, "radial_current_neg_z_final")):
        wmat = (y[:, hemi] * wt[hemi]) @ y[:, hemi].T
        got = np.imag(np.sum(np.conj(wmat @ g) * v, axis=0)) * m.r ** 2
        scale = np.abs(z[key]).max()
        np.testing.assert_allclose(got, z[key], rtol=0, atol=1e-12 * scale)


def _energy_stores():
    from ionization_gb300 import mesh

    return [mesh.Fields(), mesh.Norm(), mesh.InnerProducts(), mesh.InternalEnergyExpectationValue(),
            mesh.TotalEnergyExpectationValue()]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", CASES)
def test_device_energies_c128(cuda, kind, name):
    params, z = load_golden(name)
    sim = product_spec(kind, params, datastores=_energy_stores()).to_sim()
    sim.run()
    np.testing.assert_allclose(sim.data.internal_energy_expectation_value, z["internal_energy_expectation_value"],
                               rtol=0, atol=TOL)
    np.testing.assert_allclose(sim.data.total_energy_expectation_value, z["total_energy_expectation_value"],
                               rtol=0, atol=TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("c64", 1e-5), ("c64x", 1e-6)])
def test_device_energies_sh_complex64(cuda, precision, tol):
    params, z = load_golden("sh_energy_small")
    sim = product_spec("sh", params, precision=precision, datastores=_energy_stores()).to_sim()
    sim.run()
    np.testing.assert_allclose(sim.data.internal_energy_expectation_value, z["internal_energy_expectation_value"],
                               rtol=0, atol=tol)
    np.testing.assert_allclose(sim.data.total_energy_expectation_value, z["total_energy_expectation_value"],
                               rtol=0, atol=tol)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,rel", [("c128", 1e-9), ("c64x", 1e-4)])
def test_device_radial_current(cuda, precision, rel):
    from ionization_gb300 import mesh

    params, z = load_golden("sh_energy_small")
    store = mesh.DirectionalRadialProbabilityCurrent()
    sim = product_spec("sh", params, precision=precision,
                       datastores=[mesh.Fields(), mesh.Norm(), mesh.InnerProducts(), store]).to_sim()
    sim.run()
    for got, key in ((sim.data.radial_probability_current__pos_z[-1], "radial_current_pos_z_final"),
                     (sim.data.radial_probability_current__neg_z[-1], "radial_current_neg_z_final")):
        np.testing.assert_allclose(got, z[key], rtol=0, atol=rel * np.abs(z[key]).max())
    total = sim.data.radial_probability_current__total
    assert total.shape == (len(sim.data_times), params["r_points"])
    assert not np.isnan(total).any()


@pytest.mark.gpu
def test_velocity_gauge_sh_total_energy_is_unsupported(cuda):
    from ionization_gb300 import exceptions, mesh

    params, z = load_golden("sh_energy_small")
    params = dict(params, gauge="velocity")
    sim = product_spec("sh", params, datastores=[mesh.Norm(), mesh.InnerProducts(),
                                                 mesh.InternalEnergyExpectationValue()]).to_sim()
    sim.run()
    assert np.isfinite(sim.data.internal_energy_expectation_value).all()
    with pytest.raises(exceptions.UnsupportedMesh):
        sim.mesh.total_energy_expectation_value()


@pytest.mark.gpu
def test_expectation_kernel_imaginary_couplings(cuda):
    """ion_expectation_c128 with real and imaginary couplings along both axes
    against numpy on a random state."""
    import ctypes

    import torch

    from ionization_gb300 import _device as dev
    from ionization_gb300 import _native as nat

    rng = np.random.default_rng(7)
    na, nb = 37, 53
    g = rng.standard_normal((na, nb)) + 1j * rng.standard_normal((na, nb))
    tabs = [rng.standard_normal((na, nb)) for _ in range(3)]
    ops_np = [(tabs[0], tabs[1], tabs[2], 0), (None, tabs[1], tabs[2], nat.ION_HOP_IMAG_B | nat.ION_HOP_IMAG_A),
              (tabs[0], None, tabs[2], nat.ION_HOP_IMAG_A)]
    hops = (nat.Hop * len(ops_np))()
    keep = [dev.to_dev(t.reshape(-1)) for t in tabs]
    for q, (d, ob, oa, fl) in enumerate(ops_np):
        hops[q].diag = dev.ptr(keep[0]) if d is not None else None
        hops[q].off_b = dev.ptr(keep[1]) if ob is not None else None
        hops[q].off_a = dev.ptr(keep[2]) if oa is not None else None
        hops[q].flags = fl
    d_g = dev.to_dev(g.reshape(-1))
    nbytes = nat.value("ion_expectation_scratch_bytes", na, nb, len(ops_np))
    scratch = torch.empty(nbytes // 8, dtype=torch.float64, device=d_g.device)
    out = torch.empty(len(ops_np), dtype=torch.float64, device=d_g.device)
    nat.call("ion_expectation_c128", dev.ptr(d_g), na, nb, len(ops_np), ctypes.cast(hops, ctypes.c_void_p), 0.5,
             dev.ptr(out), dev.ptr(scratch), int(nbytes), dev.stream_ptr())
    want = [0.5 * _apply(op, g) for op in ops_np]
    np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-13, atol=1e-11)
