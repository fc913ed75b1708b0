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
