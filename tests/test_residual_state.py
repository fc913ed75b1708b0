"""The complex64 state with its stored residual (c64x), set up on the device:
psi uploaded as complex128 and split into the complex64 g and the packed
bf16x2 residual (ion_psi_split_c128), and the radial step's row-sum
remainders (ion_sh_row_lo_c64) formed with the solve's own FP32 arithmetic.
Both are checked against host restatements of the same arithmetic."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_split_matches_host_packing(cuda):
    import torch

    from ionization_gb300 import _device as dev
    from ionization_gb300 import _native as nat

    rng = np.random.default_rng(3)
    n = 50_001
    v = (rng.normal(size=n) * np.exp(rng.uniform(-60, 2, n))
         + 1j * rng.normal(size=n) * np.exp(rng.uniform(-60, 2, n)))
    v[:5] = 0
    d_in = dev.to_dev(v)
    hi = torch.empty(n, dtype=torch.complex64, device="cuda")
    lo = torch.empty(n, dtype=torch.int32, device="cuda")
    nat.call("ion_psi_split_c128", n, dev.ptr(d_in), dev.ptr(hi), dev.ptr(lo), dev.stream_ptr())
    h = hi.cpu().numpy()
    np.testing.assert_array_equal(h, v.astype(np.complex64))
    np.testing.assert_array_equal(lo.cpu().numpy(), dev.lo_pack(v - h.astype(np.complex128)))
    # and back: hi + lo carries psi to ~2^-33
    back = torch.empty(n, dtype=torch.complex128, device="cuda")
    nat.call("ion_psi_to_c128", n, dev.ptr(hi), dev.ptr(lo), dev.ptr(back), dev.stream_ptr())
    err = np.abs(back.cpu().numpy() - v) / np.maximum(np.abs(v), 1e-300)
    assert np.max(err[5:]) < 2.0 ** -31


@pytest.mark.parametrize("index", [146, 300])
def test_row_remainders_match_host_restatement(cuda, index):
    from ionization_gb300 import _device as dev
    from ionization_gb300 import batch as bm
    from ionization_gb300 import workloads as wl

    spec = wl.uneven_sh_sweep(512, steps=20, precision="c64x", subset=[index])[0]
    tab = bm._host_tables(spec)[0]
    sim = dev.ShDeviceSim(tab, "c64x")
    got = sim.d_row_lo.cpu().numpy().view(np.uint16).reshape(tab.n_l, tab.n_r)
    want = dev.bf16_bits(dev.sh_row_remainder(tab)).view(np.uint16)
    f = lambda b: (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)  # noqa: E731
    g, w = f(got), f(want)
    # the FP64 row sums differ in operation order (1e-16 of the sum), which
    # can move a remainder across a bf16 rounding boundary
    assert np.mean(got == want) > 0.999
    assert np.all(np.abs(g - w) <= 2.0 ** -7 * np.abs(w) + 1e-30)
