"""``tdma(matrix, d)`` — GPU drop-in for the reference's Cython Thomas solver.

Same call as ionization/cy.pyx:9: ``matrix`` is a scipy ``dia_matrix`` with
offsets (-1, 0, 1), ``d`` a complex128 vector; returns a new complex128 numpy
array x = matrix^-1 d.  The solve runs on the GPU (``ion_tdma_c128``); inputs
are copied to the device and the result back.  Like the reference there is no
pivoting.  Wrong dtype or dimensionality raises ValueError, as the Cython
buffer check does.

``tdma_device`` is the device-resident form (torch tensors in and out) and
``tdma_batched_device`` solves many independent systems in one launch.
"""

import numpy as np
import torch

from . import _device as dev
from . import _native as nat


def _dia_diagonals(matrix):
    data = np.asarray(matrix.data)
    offsets = list(np.asarray(matrix.offsets))
    n = matrix.shape[0]
    rows = {o: data[k] for k, o in enumerate(offsets)}
    zeros = np.zeros(n, dtype=np.complex128)
    sub = np.asarray(rows.get(-1, zeros), dtype=np.complex128)[: n - 1]
    diag = np.asarray(rows.get(0, zeros), dtype=np.complex128)
    sup = np.asarray(rows.get(1, zeros), dtype=np.complex128)[1:n]
    return sub, diag, sup


def tdma(matrix, d):
    d = np.asarray(d)
    if d.dtype != np.complex128:
        raise ValueError(f"Buffer dtype mismatch, expected 'complex128_t' but got '{d.dtype}'")
    if d.ndim != 1:
        raise ValueError(f"Buffer has wrong number of dimensions (expected 1, got {d.ndim})")
    sub, diag, sup = _dia_diagonals(matrix)
    n = d.shape[0]
    x = tdma_device(dev.to_dev(sub), dev.to_dev(diag), dev.to_dev(sup), dev.to_dev(d))
    return x.cpu().numpy()


def tdma_device(sub: torch.Tensor, diag: torch.Tensor, sup: torch.Tensor, d: torch.Tensor) -> torch.Tensor:
    n = d.shape[0]
    c128 = d.dtype == torch.complex128
    suffix = "c128" if c128 else "c64"
    x = torch.empty_like(d)
    nbytes = nat.value(f"ion_tdma_scratch_bytes_{suffix}", n)
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=d.device)
    nat.call(f"ion_tdma_{suffix}", n, dev.ptr(sub), dev.ptr(diag), dev.ptr(sup), dev.ptr(d), dev.ptr(x),
             dev.ptr(scratch), scratch.numel(), dev.stream_ptr())
    return x


def tdma_batched_device(nsys: int, n: int, sub, diag, sup, d) -> torch.Tensor:
    """nsys systems of n rows flattened back to back (the mesh layout)."""
    suffix = "c128" if d.dtype == torch.complex128 else "c64"
    x = torch.empty_like(d)
    nat.call(f"ion_tdma_batched_{suffix}", nsys, n, dev.ptr(sub), dev.ptr(diag), dev.ptr(sup), dev.ptr(d),
             dev.ptr(x), dev.stream_ptr())
    return x
