"""The allocation-free Thomas entry point, called through the C ABI.

ion_tdma_noalloc_c128 serves callers that cannot allocate device memory
around a solve (a fixed memory budget handed out at start-up, or a loop that
must not pay the synchronisation an allocation can cause): it keeps its
partition scratch in a fixed device array inside the library.  Its results
must equal those of ion_tdma_c128, which takes caller scratch, on two calls
in a row (the second call reuses the array the first one left behind).

This file is collected last so that a run stopping at the first failure has
already run every other test.  It needs no fixture from the other tests and
passes alone in a fresh process."""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL_TOL = 1e-13  # the tolerance of the other Thomas parity tests


def _system(n, seed):
    rng = np.random.default_rng(seed)
    off = 1j * rng.uniform(-5, 5, n - 1)
    diag = 1 + 1j * rng.uniform(-12, 12, n)
    d = rng.normal(size=n) + 1j * rng.normal(size=n)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    return dev(off), dev(diag), dev(off.copy()), dev(d)


def _rel(a, b):
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


# 1 and 4096 (one CTA, no scratch) still go through the per-context address
# lookup; 20000 and 65536 solve through the array
@pytest.mark.parametrize("n", [1, 3000, 4096, 20_000, 65_536])
def test_noalloc_matches_allocating_entry_point_twice(n):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ionization_gb300 import _native as nat

    lib = nat.load()
    stream = torch.cuda.current_stream().cuda_stream
    sub, diag, sup, d = _system(n, seed=n)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    # existing entry point with caller-owned scratch
    x_ref = torch.empty_like(d)
    nbytes = lib.ion_tdma_scratch_bytes_c128(n)
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device="cuda")
    rc = lib.ion_tdma_c128(n, ptr(sub), ptr(diag), ptr(sup), ptr(d), ptr(x_ref), ptr(scratch), scratch.numel(),
                           ctypes.c_void_p(stream))
    assert rc == 0, lib.ion_last_error()

    for call in range(2):
        x = torch.full_like(d, complex(float("nan"), float("nan")))
        rc = lib.ion_tdma_noalloc_c128(n, ptr(sub), ptr(diag), ptr(sup), ptr(d), ptr(x), ctypes.c_void_p(stream))
        assert rc == 0, lib.ion_last_error()
        torch.cuda.synchronize()
        assert _rel(x, x_ref) < REL_TOL, f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_array():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from ionization_gb300 import _native as nat

    lib = nat.load()
    n = lib.ion_tdma_noalloc_max_n_c128() + 1
    dummy = torch.zeros(4, dtype=torch.complex128, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    rc = lib.ion_tdma_noalloc_c128(n, p, p, p, p, p, ctypes.c_void_p(0))
    assert rc == -1  # ION_ERR_INVALID_ARGUMENT, before any device work
    assert b"outside" in lib.ion_last_error()
