"""Build and bind the oracle's C Thomas solver (``tdma.c``).

ORACLE — test infrastructure.  The shared object goes to ``oracle/_build/``
(git-ignored) and is rebuilt when ``tdma.c`` is newer.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "tdma.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_SO = os.path.join(_OUT_DIR, "liboracle_tdma.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile ``tdma.c`` with gcc (portable flags, no -march)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        tmp = _SO + f".tmp{os.getpid()}"
        subprocess.check_call(
            ["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-o", tmp, _SRC, "-lm"]
        )
        os.replace(tmp, _SO)
    return _SO


def _load():
    global _lib
    with _lock:
        if _lib is None:
            lib = ctypes.CDLL(build())
            P = ctypes.c_void_p
            I = ctypes.c_ssize_t
            lib.oracle_tdma.argtypes = [I, P, P, P, P, P]
            lib.oracle_tdma.restype = ctypes.c_int
            lib.oracle_tdma_batched.argtypes = [I, I, P, P, P, P, P]
            lib.oracle_tdma_batched.restype = ctypes.c_int
            _lib = lib
    return _lib


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def tdma(sub, diag, sup, d):
    """x = M^-1 d for one tridiagonal M (cy.tdma, ionization/cy.pyx:9-50)."""
    lib = _load()
    sub, diag, sup, d = map(_c128, (sub, diag, sup, d))
    n = d.shape[0]
    if diag.shape[0] != n or sub.shape[0] != max(n - 1, 0) or sup.shape[0] != max(n - 1, 0):
        raise ValueError("tdma: inconsistent diagonal lengths")
    x = np.empty(n, dtype=np.complex128)
    rc = lib.oracle_tdma(n, sub.ctypes.data, diag.ctypes.data, sup.ctypes.data, d.ctypes.data, x.ctypes.data)
    if rc != 0:
        raise RuntimeError("oracle_tdma failed")
    return x


def tdma_from_dia(data, d):
    """Same call shape as cy.tdma: ``data`` is a dia_matrix's (3, n) data array
    with offsets (-1, 0, 1)."""
    data = np.asarray(data)
    return tdma(data[0][:-1], data[1], data[2][1:], d)


def tdma_batched(sub, diag, sup, d):
    """Solve nsys independent systems; arrays shaped (nsys, n) / (nsys, n-1)."""
    lib = _load()
    sub, diag, sup, d = map(_c128, (sub, diag, sup, d))
    nsys, n = d.shape
    x = np.empty_like(d)
    rc = lib.oracle_tdma_batched(
        nsys, n, sub.ctypes.data, diag.ctypes.data, sup.ctypes.data, d.ctypes.data, x.ctypes.data
    )
    if rc != 0:
        raise RuntimeError("oracle_tdma_batched failed")
    return x
