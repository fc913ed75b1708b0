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


@pytest.mark.parametrize("hi_c128", [0, 1])
def test_split_rows_matches_one_row_at_a_time(cuda, hi_c128):
    """ion_psi_split_rows_c128 (all rows of a batch's initial states in one
    launch) gives what ion_psi_split_c128 gives row by row, or a plain copy
    into complex128; rows of any length, including 0 and 1, and the words
    around each destination row untouched; rows with a NULL input or a
    negative length write nothing."""
    import torch

    from ionization_gb300 import _device as dev
    from ionization_gb300 import _native as nat

    rng = np.random.default_rng(11)
    lengths = [1, 0, 257, 3000, 31, 4096, 2]
    total = sum(lengths)
    v = rng.normal(size=total) * np.exp(rng.uniform(-40, 2, total)) + 1j * rng.normal(size=total)
    d_in = dev.to_dev(v)
    hdt = torch.complex128 if hi_c128 else torch.complex64
    gap = 3  # untouched elements between destination rows
    extra = 8  # the target of rows that must be skipped (NULL input, negative length)
    hi = torch.full((total + gap * len(lengths) + extra,), 7.0, dtype=hdt, device="cuda")
    lo = torch.full((total + gap * len(lengths) + extra,), -1, dtype=torch.int32, device="cuda")
    table, o_in, o_out = [], 0, 0
    for n in lengths:
        table.append((d_in.data_ptr() + 16 * o_in, hi.data_ptr() + hi.element_size() * o_out,
                      0 if hi_c128 else lo.data_ptr() + 4 * o_out, n))
        o_in += n
        o_out += n + gap
    end_hi, end_lo = hi.data_ptr() + hi.element_size() * o_out, lo.data_ptr() + 4 * o_out
    table.insert(2, (0, end_hi, end_lo, extra))
    table.append((d_in.data_ptr(), end_hi, end_lo, -3))
    d_table = torch.tensor(table, dtype=torch.int64, device="cuda")
    assert nat.call("ion_psi_split_rows_c128", len(table), d_table.data_ptr(), hi_c128, dev.stream_ptr()) == 0
    torch.cuda.synchronize()
    keep = np.concatenate([np.r_[np.ones(n, bool), np.zeros(gap, bool)] for n in lengths] + [np.zeros(extra, bool)])
    h, w = hi.cpu().numpy(), lo.cpu().numpy()
    if hi_c128:
        np.testing.assert_array_equal(h[keep], v)
    else:
        np.testing.assert_array_equal(h[keep], v.astype(np.complex64))
        np.testing.assert_array_equal(w[keep], dev.lo_pack(v - v.astype(np.complex64).astype(np.complex128)))
    np.testing.assert_array_equal(h[~keep], 7.0)
    np.testing.assert_array_equal(w[~keep], -1)
    assert nat.call("ion_psi_split_rows_c128", 0, None, hi_c128, dev.stream_ptr()) == 0
    with pytest.raises(nat.IonError):
        nat.call("ion_psi_split_rows_c128", 3, None, hi_c128, dev.stream_ptr())


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
