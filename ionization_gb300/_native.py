"""ctypes binding of the C ABI declared in ``include/ionization_gb300.h``.

The library is the only compute path of this package: if it is missing or
fails to load, every entry point raises ``NativeLibraryError`` (there is no
CPU fallback).  Structures below mirror the header field by field.
"""

import ctypes
import os
import threading

from . import _build

c_i32, c_i64, c_f32, c_f64, c_vp = (
    ctypes.c_int32,
    ctypes.c_int64,
    ctypes.c_float,
    ctypes.c_double,
    ctypes.c_void_p,
)

ION_OK = 0
ION_LINE_ADI = 0
ION_LINE_SPLIT = 1
ION_LINE_FFT = 2
ION_SH_REFINE = 1
ION_SH_VELOCITY = 2
ION_SH_ONLY_VELOCITY = 4
ION_SH_COUPLED = 8
ION_GAUGE_LENGTH = 0
ION_ADI_STRIDED_FIRST = 0
ION_ADI_CONTIG_FIRST = 1
ION_ADI_PASS_STRIDED = 0
ION_ADI_PASS_CONTIG = 1
ION_GAUGE_VELOCITY = 1
ION_LINE_RESIDUAL = 1
ION_LINE_HAS_FFT = 2
ION_HOP_IMAG_B = 1
ION_HOP_IMAG_A = 2
ION_HOP_WRAP_B = 4
ION_MAX_HOPS = 4


class NativeLibraryError(RuntimeError):
    pass


class IonError(RuntimeError):
    def __init__(self, fn, code, msg):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


class ShSim(ctypes.Structure):
    _fields_ = [
        ("g", c_vp),
        ("n_r", c_i32),
        ("n_l", c_i32),
        ("t", c_i64),
        ("t_final", c_i64),
        ("store_every", c_i64),
        ("hd", c_vp),
        ("hoff", c_vp),
        ("rq", c_vp),
        ("cl", c_vp),
        ("mask", c_vp),
        ("tau", c_vp),
        ("efield", c_vp),
        ("kinv32", c_vp),
        ("cent32", c_vp),
        ("hoff32", c_vp),
        ("rq32", c_vp),
        ("cl32", c_vp),
        ("mask32", c_vp),
        ("corr0_32", c_f32),
        ("n_states", c_i32),
        ("state_l", c_vp),
        ("state_g", c_vp),
        ("weight", c_f64),
        ("out_norm", c_vp),
        ("out_ip", c_vp),
        ("partials", c_vp),
        ("n_tiles", c_i32),
        ("gauge", c_i32),
        ("g_lo", c_vp),
        ("h2r", c_vp),
        ("h2r32", c_vp),
        ("row_lo", c_vp),
        ("kinv", c_vp),
        ("cent", c_vp),
        ("corr0", c_f64),
        ("spike_s", c_vp),
        ("spike_t", c_vp),
        ("edge", c_vp),
        ("hcross", c_f64),
        ("state_real", c_i32),
        ("pad3_", c_i32),
    ]


class ShPlan(ctypes.Structure):
    _fields_ = [
        ("sims", c_vp),
        ("n_sims", c_i32),
        ("max_n_l", c_i32),
        ("max_n_r", c_i32),
        ("flags", c_i32),
        ("cn_items", c_vp),
        ("n_cn_items", c_i32),
        ("cn_threads", c_i32),
        ("rot_items", c_vp),
        ("n_rot_items", c_i32),
        ("rot_rows", c_i32),
        ("cn_rows", c_i32),
        ("n_cn_buckets", c_i32),
        ("cn_bucket_end", c_i32 * 8),
        ("cn_bucket_threads", c_i32 * 8),
        ("cn_bucket_rows", c_i32 * 8),
    ]


class LineSim(ctypes.Structure):
    _fields_ = [
        ("g", c_vp),
        ("n", c_i32),
        ("method", c_i32),
        ("t", c_i64),
        ("t_final", c_i64),
        ("store_every", c_i64),
        ("hd", c_vp),
        ("hoff", c_vp),
        ("zq", c_vp),
        ("mask", c_vp),
        ("tau", c_vp),
        ("efield", c_vp),
        ("hd32", c_vp),
        ("hoff32", c_vp),
        ("zq32", c_vp),
        ("mask32", c_vp),
        ("n_states", c_i32),
        ("gauge", c_i32),
        ("state_g", c_vp),
        ("weight", c_f64),
        ("out_norm", c_vp),
        ("out_ip", c_vp),
        ("vstat", c_vp),
        ("kin", c_vp),
        ("twiddle", c_vp),
        ("vstat32", c_vp),
        ("g_lo", c_vp),
        ("vcoef", c_f64),
        ("hd_lo32", c_vp),
        ("hoff_lo32", c_vp),
    ]


class LinePlan(ctypes.Structure):
    _fields_ = [
        ("sims", c_vp),
        ("n_sims", c_i32),
        ("max_n", c_i32),
        ("threads", c_i32),
        ("cluster", c_i32),
        ("flags", c_i32),
        ("pad2_", c_i32),
    ]


class Hop(ctypes.Structure):
    _fields_ = [
        ("diag", c_vp),
        ("off_b", c_vp),
        ("off_a", c_vp),
        ("flags", c_i32),
        ("pad_", c_i32),
    ]


class PsiRow(ctypes.Structure):
    _fields_ = [
        ("in", c_vp),  # (a Python keyword: set with setattr or the numpy view)
        ("hi", c_vp),
        ("lo", c_vp),
        ("n", c_i64),
    ]


class CylMesh(ctypes.Structure):
    _fields_ = [
        ("n_z", c_i32),
        ("n_rho", c_i32),
        ("hz_d", c_vp),
        ("hz_off", c_vp),
        ("hr_d", c_vp),
        ("hr_off", c_vp),
        ("zq", c_vp),
        ("mask", c_vp),
        ("tau", c_vp),
        ("efield", c_vp),
        ("hz_off_col", c_vp),
        ("order", c_i32),
        ("pad_", c_i32),
        ("hr_off_row", c_vp),
        ("zq_pt", c_vp),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "ion_last_error": (ctypes.c_char_p, []),
    "ion_version": (ctypes.c_int, []),
    "ion_tdma_scratch_bytes_c128": (c_i64, [c_i64]),
    "ion_tdma_scratch_bytes_c64": (c_i64, [c_i64]),
    "ion_tdma_c128": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "ion_tdma_c64": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i64, c_vp]),
    "ion_tdma_noalloc_c128": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_tdma_noalloc_max_n_c128": (c_i64, []),
    "ion_tdma_batched_c128": (ctypes.c_int, [c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_tdma_batched_c64": (ctypes.c_int, [c_i64, c_i64, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_tdma_batched_max_n_c128": (c_i64, []),
    "ion_tdma_batched_max_n_c64": (c_i64, []),
    "ion_sh_split_run_c128": (ctypes.c_int, [ctypes.POINTER(ShPlan), c_i64, c_vp]),
    "ion_sh_split_run_c64": (ctypes.c_int, [ctypes.POINTER(ShPlan), c_i64, c_vp]),
    "ion_sh_split_phase_c128": (ctypes.c_int, [ctypes.POINTER(ShPlan), ctypes.c_int, c_vp]),
    "ion_sh_split_phase_c64": (ctypes.c_int, [ctypes.POINTER(ShPlan), ctypes.c_int, c_vp]),
    "ion_sh_reduce_c128": (ctypes.c_int, [ctypes.POINTER(ShPlan), c_vp]),
    "ion_sh_reduce_c64": (ctypes.c_int, [ctypes.POINTER(ShPlan), c_vp]),
    "ion_sh_max_n_r_c128": (c_i64, []),
    "ion_sh_max_n_r_c64": (c_i64, []),
    "ion_line_run_c128": (ctypes.c_int, [ctypes.POINTER(LinePlan), c_i64, c_vp]),
    "ion_line_run_c64": (ctypes.c_int, [ctypes.POINTER(LinePlan), c_i64, c_vp]),
    "ion_line_reduce_c128": (ctypes.c_int, [ctypes.POINTER(LinePlan), c_vp]),
    "ion_line_reduce_c64": (ctypes.c_int, [ctypes.POINTER(LinePlan), c_vp]),
    "ion_line_max_n_c128": (c_i64, []),
    "ion_line_max_n_c64": (c_i64, []),
    "ion_line_max_n_c64x": (c_i64, []),
    "ion_cyl_adi_run_c128": (ctypes.c_int, [ctypes.POINTER(CylMesh), c_vp, c_vp, c_i64, c_i64, c_vp]),
    "ion_sh_row_lo_c64": (ctypes.c_int, [ctypes.POINTER(ShPlan), c_vp]),
    "ion_psi_split_c128": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp]),
    "ion_psi_split_rows_c128": (ctypes.c_int, [c_i64, c_vp, c_i32, c_vp]),
    "ion_cyl_adi_pass_c128": (ctypes.c_int, [ctypes.POINTER(CylMesh), c_vp, c_vp, c_i64, c_i32, c_i32, c_vp]),
    "ion_cyl_max_points_c128": (c_i64, []),
    "ion_cyl_adi_run_c64": (ctypes.c_int, [ctypes.POINTER(CylMesh), c_vp, c_vp, c_i64, c_i64, c_vp]),
    "ion_cyl_adi_pass_c64": (ctypes.c_int, [ctypes.POINTER(CylMesh), c_vp, c_vp, c_i64, c_i32, c_i32, c_vp]),
    "ion_cyl_max_points_c64": (c_i64, []),
    "ion_tridiag_eig_scratch_doubles": (c_i64, [c_i32, c_i32]),
    "ion_tridiag_count_below": (ctypes.c_int, [c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_tridiag_eigvals": (ctypes.c_int, [c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp]),
    "ion_tridiag_eigvecs": (ctypes.c_int, [c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_reduce_scratch_bytes": (c_i64, [c_i64, c_i32]),
    "ion_reduce_c128": (ctypes.c_int, [c_i64, c_vp, c_i32, c_vp, c_f64, c_vp, c_vp, c_vp, c_vp]),
    "ion_reduce_c64": (ctypes.c_int, [c_i64, c_vp, c_i32, c_vp, c_f64, c_vp, c_vp, c_vp, c_vp]),
    "ion_psi_to_c128": (ctypes.c_int, [c_i64, c_vp, c_vp, c_vp, c_vp]),
    "ion_weighted_norms_scratch_bytes": (c_i64, [c_i64, c_i32]),
    "ion_weighted_norms_c128": (ctypes.c_int, [c_i64, c_vp, c_i32, c_vp, c_f64, c_vp, c_vp, c_i64, c_vp]),
    "ion_weighted_norms_c64": (ctypes.c_int, [c_i64, c_vp, c_vp, c_i32, c_vp, c_f64, c_vp, c_vp, c_i64, c_vp]),
    "ion_expectation_scratch_bytes": (c_i64, [c_i32, c_i32, c_i32]),
    "ion_expectation_c128": (ctypes.c_int, [c_vp, c_i32, c_i32, c_i32, c_vp, c_f64, c_vp, c_vp, c_i64, c_vp]),
    "ion_expectation_c64": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_f64, c_vp, c_vp, c_i64, c_vp]),
    "ion_sh_radial_current_c128": (ctypes.c_int, [c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_sh_radial_current_c64": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "ion_sh_observables_scratch_bytes": (c_i64, [c_i32, c_i32, c_i32]),
    "ion_sh_observables_c128": (ctypes.c_int, [c_vp, c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_f64, c_vp, c_vp,
                                                c_i64, c_vp]),
    "ion_sh_observables_c64": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_vp, c_vp, c_i32, c_vp, c_f64, c_vp,
                                               c_vp, c_i64, c_vp]),
}

_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
            try:
                _build.build()
            except Exception as e:  # noqa: BLE001
                raise NativeLibraryError(f"cannot build the CUDA library: {e}") from e
        if not os.path.exists(path):
            raise NativeLibraryError(f"CUDA library missing: {path}")
        try:
            lib = ctypes.CDLL(path)
        except OSError as e:
            raise NativeLibraryError(f"cannot load {path}: {e}") from e
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name, *args):
    """Call an int-returning entry point and raise IonError on failure."""
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != ION_OK:
        msg = lib.ion_last_error().decode(errors="replace")
        raise IonError(name, rc, msg)
    return rc


def value(name, *args):
    return getattr(load(), name)(*args)


def exported_symbols():
    return list(_SIGS)
