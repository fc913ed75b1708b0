"""Line Fourier split-step (FourierSplitOperator).

The reference has no Fourier method, so the oracle (oracle/mesh.py, a
numpy.fft statement of the step) is pinned analytically: with no potential the
split-step is exact for band-limited wavefunctions, and a free Gaussian must
follow its closed-form spreading.  The device's in-place transform order
(radix-4 decimation in frequency with a bit-reversed spectrum, exact inverse
butterflies in reverse order) is checked on the host against numpy.fft with a
model of the same stage sequence.  The GPU tests then compare the CUDA path
with the oracle through the C ABI (complex128: relative L2 <= 1e-10)."""

import copy

import numpy as np
import pytest

from oracle import mesh as om
from oracle import physics as ph

from .conftest import load_golden, rel_l2
from .specs import product_spec


# ------------------------------------------------------------------ host model of the device stage order


def _dif4(x, lq, tw):
    n = len(x)
    q = 1 << lq
    s = n >> (lq + 2)
    for b in range(n >> 2):
        k = b & (q - 1)
        i0 = ((b >> lq) << (lq + 2)) + k
        a0, a1, a2, a3 = x[i0], x[i0 + q], x[i0 + 2 * q], x[i0 + 3 * q]
        t0, t1, t2, t3 = a0 + a2, a0 - a2, a1 + a3, -1j * (a1 - a3)
        x[i0] = t0 + t2
        x[i0 + q] = (t0 - t2) * tw[2 * k * s]
        x[i0 + 2 * q] = (t1 + t3) * tw[k * s]
        x[i0 + 3 * q] = (t1 - t3) * tw[3 * k * s]


def _dif4_inverse(x, lq, tw):
    n = len(x)
    q = 1 << lq
    s = n >> (lq + 2)
    for b in range(n >> 2):
        k = b & (q - 1)
        i0 = ((b >> lq) << (lq + 2)) + k
        y0 = x[i0]
        u2 = x[i0 + q] * np.conj(tw[2 * k * s])
        u1 = x[i0 + 2 * q] * np.conj(tw[k * s])
        u3 = x[i0 + 3 * q] * np.conj(tw[3 * k * s])
        t0, t2, t1, t3 = y0 + u2, y0 - u2, u1 + u3, 1j * (u1 - u3)
        x[i0], x[i0 + 2 * q], x[i0 + q], x[i0 + 3 * q] = t0 + t1, t0 - t1, t2 + t3, t2 - t3


def _pairs(x):
    a, b = x[0::2].copy(), x[1::2].copy()
    x[0::2], x[1::2] = a + b, a - b


def _bitrev(n):
    bits = n.bit_length() - 1
    idx = np.arange(n)
    rev = np.zeros(n, dtype=np.int64)
    for b in range(bits):
        rev |= ((idx >> b) & 1) << (bits - 1 - b)
    return rev


def _forward(x):
    n = len(x)
    lg = n.bit_length() - 1
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    for lq in range(lg - 2, -1, -2):
        _dif4(x, lq, tw)
    if lg & 1:
        _pairs(x)


def _inverse(x):
    n = len(x)
    lg = n.bit_length() - 1
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    if lg & 1:
        _pairs(x)
    for lq in range(lg & 1, lg - 1, 2):
        _dif4_inverse(x, lq, tw)


@pytest.mark.parametrize("n", [2, 4, 8, 32, 512, 2048])
def test_stage_order_gives_bit_reversed_spectrum_and_exact_inverse(n):
    rng = np.random.default_rng(n)
    x0 = rng.normal(size=n) + 1j * rng.normal(size=n)
    x = x0.copy()
    _forward(x)
    np.testing.assert_allclose(x, np.fft.fft(x0)[_bitrev(n)], rtol=0, atol=1e-11 * np.abs(x0).sum())
    _inverse(x)
    np.testing.assert_allclose(x / n, x0, rtol=0, atol=1e-13 * np.abs(x0).max())


def test_host_kinetic_table_is_bit_reversed():
    """fourier_tables places E_kin(k_j) at the bit-reversed index of j."""
    from ionization_gb300 import mesh, potentials, states

    spec = mesh.LineSpecification(
        "t", z_bound=20.0, z_points=64, test_mass=1.0, initial_state=states.GaussianState(width=1.0),
        internal_potential=potentials.SoftCoulombPotential(softening_distance=1.0),
        evolution_method=mesh.FourierSplitOperator(), time_initial=0, time_final=0.1, time_step=0.05,
    )
    spec.host_only = True
    sim = spec.to_sim()
    V, kin, tw = sim.mesh.operators.fourier_tables(sim.mesh)
    k = 2 * np.pi * np.fft.fftfreq(64, d=sim.mesh.delta_z)
    np.testing.assert_array_equal(kin[_bitrev(64)], k ** 2 / 2)
    np.testing.assert_allclose(tw, np.exp(-2j * np.pi * np.arange(64) / 64), rtol=0, atol=1e-15)
    assert V.shape == (64,) and np.all(V < 0)


# ------------------------------------------------------------------ oracle pin


def test_oracle_free_gaussian_matches_closed_form():
    """V = 0, no field: psi(z, t) = (1 + i t / s^2)^(-1/2) exp(-z^2 / (2 s^2 (1 + i t / s^2)))."""
    zero = ph.CosSquaredPulse(amplitude=0.0, omega_carrier=1.0, number_of_cycles=1, phase=0.0, pulse_center=0.0)
    st = om.LineLength(512, 40.0, 1.0, 1.0, zero, None, "FourierSplitOperator", gaussian_width=1.0)
    st.V = np.zeros_like(st.V)
    g0 = ph.gaussian(st.z, 1.0)
    c = st.g[256] / g0[256]
    times = om.get_times(0.0, 5.0, 0.05)
    om.run(st, times, -1)
    t = times[-1]
    a = 1 + 1j * t
    exact = c * a ** -0.5 * np.exp(-(st.z ** 2) / (2 * a))
    assert rel_l2(st.g, exact) < 1e-12


def _fft_params(name, n=None, time_final=None):
    params, _ = load_golden(name)
    params = copy.deepcopy(params)
    params["method"] = "FourierSplitOperator"
    if n is not None:
        params["z_points"] = n
    if time_final is not None:
        params["time_final"] = time_final
    return params


def test_oracle_fourier_conserves_norm_without_mask():
    params = _fft_params("line_split_small", time_final=5.0)
    params["mask"] = None
    out = om.run_from_params("line", params)
    assert np.max(np.abs(out["norm"] - out["norm"][0])) < 1e-12


# ------------------------------------------------------------------ GPU parity


FFT_CASES = [("line_split_small", None, None), ("line_split_small", 2048, None), ("line_cfg1_full", None, 20.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,tf", FFT_CASES)
def test_fourier_c128_matches_oracle(cuda, name, n, tf):
    params = _fft_params(name, n, tf)
    want = om.run_from_params("line", params)
    sim = product_spec("line", params).to_sim()
    sim.run()
    assert rel_l2(sim.mesh.g, want["g_final"]) < 1e-10
    np.testing.assert_allclose(sim.data.norm, want["norm"], rtol=0, atol=1e-10)
    ips = np.array([sim.data.inner_products[s] for s in sim.spec.test_states])
    np.testing.assert_allclose(ips, want["inner_products"], rtol=0, atol=1e-10)


@pytest.mark.gpu
def test_fourier_c64_population_error(cuda):
    params = _fft_params("line_split_small")
    want = om.run_from_params("line", params)
    sim = product_spec("line", params, precision="c64").to_sim()
    sim.run()
    p64 = sim.data.initial_state_overlap[-1]
    p128 = abs(want["inner_products"][0][-1]) ** 2
    print(f"fourier c64: |P_c64 - P_c128| = {abs(p64 - p128):.2e}")
    assert abs(p64 - p128) < 1e-4
    assert rel_l2(sim.mesh.g, want["g_final"]) < 1e-3


@pytest.mark.gpu
def test_fourier_and_crank_nicolson_share_one_plan(cuda):
    """Lines of different methods and sizes advance in one launch."""
    from ionization_gb300 import _device as dev

    cases = [_fft_params("line_split_small"), _fft_params("line_split_small", 1024), load_golden("line_split_small")[0]]
    sims = [product_spec("line", p).to_sim() for p in cases]
    batch = dev.LineBatch("c128", [s.mesh._dsim for s in sims], spread=1)
    assert len(batch.plans) == 1
    steps = sims[0].mesh._dsim.t_final
    batch.run(steps)
    for p, s in zip(cases, sims):
        want = om.run_from_params("line", p)
        assert rel_l2(s.mesh._dsim.psi_host(), want["g_final"]) < 1e-10
