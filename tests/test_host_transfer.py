"""Host side of the batch transfers, on the CPU (the device buffer replaced by
a host tensor): the upload packing (``_Arena``) puts every array where its
view says, aligns the first array of each kind, places an array object added
twice once, and the readback (``_host_copy``) returns the tensor's values,
for small buffers and for large ones touched by several threads first."""

import numpy as np
import pytest
import torch

from ionization_gb300 import _device as dev


@pytest.fixture
def host_device(monkeypatch):
    monkeypatch.setattr(dev, "device", lambda: torch.device("cpu"))


def _view(v):
    return v.tensor if isinstance(v, dev._DevSlice) else v


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.complex128])
def test_arena_views_hold_their_arrays(host_device, dtype):
    rng = np.random.default_rng(5)
    ar = dev._Arena(dtype)
    arrays = {}
    for i in range(40):
        for kind, n in (("a", 1 + 7 * i), ("b", 300 + i), ("c", 16)):
            x = rng.normal(size=n).astype(dtype)
            arrays[(i, kind)] = x
    shared = rng.normal(size=33).astype(dtype)
    for kind in ("a", "b", "c"):  # kind by kind, as ShDeviceSim.bulk adds them
        for i in range(40):
            ar.add((i, kind), arrays[(i, kind)], align=(i == 0))
    for i in range(40):
        ar.add((i, "s"), shared, align=(i == 0))
    views = ar.upload(tensors=("b",))
    assert len(views) == 4 * 40
    for key, x in arrays.items():
        v = views[key]
        assert isinstance(v, torch.Tensor) == (key[1] == "b")
        np.testing.assert_array_equal(_view(v).numpy(), x)
    # the shared array is placed once: every key views the same elements
    ptrs = {views[(i, "s")].data_ptr() for i in range(40)}
    assert len(ptrs) == 1
    np.testing.assert_array_equal(_view(views[(7, "s")]).numpy(), shared)
    # the first array of each kind starts on a 64-byte boundary of the buffer
    base = views[(0, "b")].data_ptr() - views[(0, "b")].storage_offset() * views[(0, "b")].element_size()
    for kind in ("a", "b", "c", "s"):
        assert (views[(0, kind)].data_ptr() - base) % 64 == 0
    # a kind's arrays follow one another: at most one run per kind (kinds
    # that meet without an alignment gap merge), each placed array in one run
    runs = ar.runs()
    assert len(runs) <= 4
    assert sum(len(arrs) for _, arrs in runs) == len(ar.placed) == 3 * 40 + 1


@pytest.mark.parametrize("n", [0, 5, 3_000_000])
def test_host_copy_returns_the_values(n):
    t = torch.arange(n, dtype=torch.float64) * 0.5 - 3.0
    if n:
        t = t.reshape(-1, 5) if n % 5 == 0 else t
    out = dev._host_copy(t)
    assert out.shape == tuple(t.shape) and out.dtype == np.float64
    np.testing.assert_array_equal(out, t.numpy())
    c = torch.complex(t, -t)
    np.testing.assert_array_equal(dev._host_copy(c), c.numpy())


def test_lazy_array_forms_once_and_reads_like_its_array():
    from ionization_gb300.core import LazyArray

    calls = []

    def make():
        calls.append(1)
        return np.arange(12, dtype=np.float64).reshape(3, 4)

    a = LazyArray(make)
    assert not calls
    np.testing.assert_array_equal(np.asarray(a), make())
    assert np.asarray(a, dtype=np.float32).dtype == np.float32
    assert a.shape == (3, 4) and a.dtype == np.float64 and len(a) == 3
    assert a[1, 2] == 6.0 and a.reshape(-1)[5] == 5.0
    np.testing.assert_array_equal(np.asarray(a, dtype=np.complex128).real, make())
    assert len(calls) == 3  # one inside LazyArray, two by the test itself


@pytest.mark.parametrize("precision", ["c128", "c64x", "c64"])
def test_lazy_sh_tables_upload_what_eager_ones_do(precision):
    """The spherical-harmonic host tables form the (l, r) diagonal and the
    full initial psi only when read: what a simulation uploads equals what
    the same tables with both formed up front give, and the complex64 forms
    never form the diagonal."""
    import dataclasses

    from ionization_gb300 import batch as bm
    from ionization_gb300 import workloads as wl
    from ionization_gb300.core import LazyArray

    spec = wl.sh_spec("lazy", 160, 9, 0.05, 0.1, 2, 0.3, 12, precision=precision, mask_width=0.4 * wl.DR * 160)
    tab = bm._host_tables(spec)[0]
    assert isinstance(tab.hd, LazyArray) and isinstance(tab.g0, LazyArray)
    got = dev._sh_host_arrays(tab, precision)
    assert (tab.hd._value is None) == (precision != "c128")
    eager = dataclasses.replace(tab, hd=np.array(tab.hd), g0=np.array(tab.g0), g0_rows=None, g0_row_data=None)
    want = dev._sh_host_arrays(eager, precision)
    assert got.keys() == want.keys()
    for k in got:
        if want[k] is None:
            assert got[k] is None, k
        else:
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    np.testing.assert_array_equal(dev.sh_nonzero_rows(tab), dev.sh_nonzero_rows(eager))
