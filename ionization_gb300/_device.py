"""Device-resident simulation state and the plans handed to the C ABI.

PyTorch provides device memory and the stream; every kernel is ours, called
through ``_native``.  A *batch* owns the psi buffers, coefficient tables and
data buffers of any number of simulations and builds the descriptor array
(``ion_sh_sim`` / ``ion_line_sim``) and work lists that one launch sweeps.
The plain meshes are batches of one; the batched and served forms put many
simulations of different sizes in one batch.
"""

import concurrent.futures
import ctypes
import dataclasses
import os
from typing import List, Optional

import numpy as np
import torch

from . import _native as nat
from .core import Precision


class DeviceUnavailable(RuntimeError):
    pass


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise DeviceUnavailable("ionization_gb300 needs a CUDA device; none is available")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def to_dev(a, dtype=None) -> torch.Tensor:
    a = np.array(a, dtype=dtype, copy=True, order="C")
    return torch.from_numpy(a).to(device(), non_blocking=False)


def ptr(t) -> Optional[int]:
    """Device address of a tensor or of a ``_DevSlice`` (None: NULL)."""
    return None if t is None else t.data_ptr()


class _DevSlice:
    """Part of a bulk device buffer held as (buffer, element offset, shape):
    the descriptors need only its address, and a torch view (``tensor``) is
    made on first use (thousands of small views cost tens of ms to make)."""

    __slots__ = ("buf", "off", "shape", "_t")

    def __init__(self, buf: torch.Tensor, off: int, shape):
        self.buf, self.off, self.shape, self._t = buf, int(off), tuple(shape), None

    def data_ptr(self) -> int:
        return self.buf.data_ptr() + self.off * self.buf.element_size()

    def numel(self) -> int:
        return int(np.prod(self.shape))

    def element_size(self) -> int:
        return self.buf.element_size()

    @property
    def tensor(self) -> torch.Tensor:
        if self._t is None:
            self._t = self.buf[self.off:self.off + self.numel()].view(self.shape)
        return self._t


def _tensor(t):
    return t.tensor if isinstance(t, _DevSlice) else t


def n_data_slots(t_final: int, store_every: int) -> int:
    """Number of data times of MeshSimulation.__init__ (sims.py:84-90)."""
    if store_every >= 1:
        return t_final // store_every + 1 + (1 if t_final % store_every != 0 else 0)
    return 2 if t_final > 0 else 1


def data_slot(t: int, t_final: int, store_every: int) -> int:
    if store_every >= 1:
        return t // store_every if t % store_every == 0 else t_final // store_every + 1
    return 0 if t == 0 else 1


def is_data_time(t: int, t_final: int, store_every: int) -> bool:
    return t == 0 or t == t_final or (store_every >= 1 and t % store_every == 0)


def complex_dtype(precision) -> torch.dtype:
    return torch.complex128 if Precision(precision) == Precision.C128 else torch.complex64


def _round32(x: int) -> int:
    return (x + 31) // 32 * 32


def _pad16(a) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    out = np.zeros((a.size + 16) // 16 * 16, dtype=np.float64)
    out[: a.size] = a
    return out


# ==========================================================================
# spherical-harmonic split operator
# ==========================================================================


@dataclasses.dataclass
class ShTables:
    """Host FP64 inputs of one spherical-harmonic simulation."""

    n_r: int
    n_l: int
    hd: np.ndarray  # [n_l * n_r] internal diagonal, C order (may be a LazyArray)
    hoff: np.ndarray  # [n_r - 1]
    rq: np.ndarray  # [n_r]
    cl: np.ndarray  # [n_l]
    mask: Optional[np.ndarray]  # [n_r]
    tau: np.ndarray  # [t_final + 1]
    efield: np.ndarray  # [t_final + 1]
    kinv: np.ndarray  # [n_r]  -2p beta(j) + V(r_j)
    cent: np.ndarray  # [n_r]
    corr0: float
    state_l: List[int]
    state_g: np.ndarray  # [n_states, n_r] complex128, or float64 for real states
    weight: float
    g0: np.ndarray  # [n_l, n_r] complex128 (may be a LazyArray)
    t0: int
    t_final: int
    store_every: int
    # velocity gauge: rq holds hbar (q/m) / r_j, efield the vector potential
    # A(times[t]) and h2r [n_r - 1] the r factor of the h2 blocks
    gauge: int = 0
    h2r: Optional[np.ndarray] = None
    # the l rows of g0 that are not zero (None: find them); only those rows
    # are uploaded, the rest are zeroed on the device
    g0_rows: Optional[np.ndarray] = None
    # [len(g0_rows), n_r] complex128: those rows' values (None: read g0)
    g0_row_data: Optional[np.ndarray] = None
    # kinetic_energy_from_hamiltonian: the coupling between the last r of
    # each l and the first r of the next (None: the lines are independent)
    hcross: Optional[float] = None


SH_ROT_ROWS = 32


SH_ROWS_CHOICES = {Precision.C128: (8, 4), Precision.C64: (16, 8), Precision.C64X: (8, 4, 16)}  # default first
SH_MAX_LINE_THREADS = 512  # threads of one radial-solve CTA


def sh_max_line_threads(precision, rows: int) -> int:
    """Largest radial-solve CTA at ``rows`` rows per thread: the complex64
    4-row variant runs in 64 registers and so takes up to 1024 threads."""
    return 1024 if Precision(precision) != Precision.C128 and rows == 4 else SH_MAX_LINE_THREADS


def sh_default_rows(precision, max_n_r: int) -> int:
    """Rows per thread of the radial solve when none is asked for: the first
    choice whose CTA holds the longest line of the batch."""
    for rows in SH_ROWS_CHOICES[Precision(precision)]:
        if (max_n_r + rows - 1) // rows <= sh_max_line_threads(precision, rows):
            return rows
    return max(SH_ROWS_CHOICES[Precision(precision)])


def sh_line_threads(n_r: int, precision, rows: int = 0) -> int:
    maxm = rows or SH_ROWS_CHOICES[Precision(precision)][0]
    return (n_r + maxm - 1) // maxm  # the line is padded to whole chunks


def sh_bucket_sizes(n_rs, precision, rows: int) -> np.ndarray:
    """The radial-solve CTA size of each simulation's lines: its threads at
    ``rows`` rows per thread, rounded up to a granularity (32, doubled while
    there would be more than 8 distinct sizes).  Lines of equal size form one
    bucket, one launch."""
    need = [_round32(sh_line_threads(n, precision, rows)) for n in n_rs]
    gran = 32
    while len({(n + gran - 1) // gran * gran for n in need}) > 8:
        gran *= 2
    return np.array([(n + gran - 1) // gran * gran for n in need], dtype=np.int64)


def lo_pack(lo) -> np.ndarray:
    """The stored residual of a complex64 state from its complex value: one
    32-bit word a point (int32 holding the bits), the real part's bf16 in the
    low half and the imaginary part's in the high half, each rounded to
    nearest even as the device's cvt.rn.bf16x2.f32 does."""
    c = np.ascontiguousarray(np.asarray(lo, dtype=np.complex64))
    u = c.view(np.uint32).reshape(c.shape + (2,)).astype(np.uint64)
    r = ((u + np.uint64(0x7FFF) + ((u >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)) & np.uint64(0xFFFF)
    return (r[..., 0] | (r[..., 1] << np.uint64(16))).astype(np.uint32).view(np.int32)


def lo_unpack(w) -> np.ndarray:
    """The complex128 value of packed residual words (``lo_pack``)."""
    u = np.ascontiguousarray(np.asarray(w)).view(np.uint32)
    re = (u << np.uint32(16)).view(np.float32).astype(np.float64)
    im = (u & np.uint32(0xFFFF0000)).view(np.float32).astype(np.float64)
    return re + 1j * im


def _lo32(a) -> np.ndarray:
    """The FP32 low part of FP64 values: float32(a - float32(a))."""
    a = np.asarray(a, dtype=np.float64)
    return (a - a.astype(np.float32).astype(np.float64)).astype(np.float32)


def bf16_bits(x) -> np.ndarray:
    """FP64 values rounded to FP32 and then to bf16 (nearest even), as int16 bits."""
    u = np.ascontiguousarray(np.asarray(x, dtype=np.float64).astype(np.float32)).view(np.uint32).astype(np.uint64)
    r = ((u + np.uint64(0x7FFF) + ((u >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)) & np.uint64(0xFFFF)
    return r.astype(np.uint16).view(np.int16)


def sh_row_remainder(tab: "ShTables") -> np.ndarray:
    """[n_l, n_r] FP64, a host restatement of ion_sh_row_lo_c64: the exact row
    sum of the radial step's coefficients, tau (H_ii + H_i,i-1 + H_i,i+1) from
    the FP64 tables, minus the sum of the FP32 coefficients the complex64
    radial solve forms for that row: bd = fl(tau32 fl(fma(l(l+1), cent32,
    kinv32)) [+ corr0 at (0, 0)]), bo = fl(tau32 hoff32).  Every FP32
    operation is reproduced in FP64 and rounded once (the products and sums
    of FP32 values it rounds are exact in FP64)."""
    f32 = lambda v: np.asarray(v, np.float64).astype(np.float32).astype(np.float64)  # noqa: E731
    nl, nr = int(tab.n_l), int(tab.n_r)
    tau64 = float(tab.tau[1]) if len(tab.tau) > 1 else 0.0
    tau32 = float(np.float32(tau64))
    ll1 = (np.arange(nl, dtype=np.float64) * (np.arange(nl, dtype=np.float64) + 1))[:, None]
    h32 = f32(f32(tab.kinv)[None, :] + ll1 * f32(tab.cent)[None, :])
    h32[0, 0] = f32(h32[0, 0] + f32(tab.corr0))
    bd32 = f32(tau32 * h32)
    bo32 = np.zeros(nr + 1)
    bo32[1:nr] = f32(tau32 * f32(tab.hoff))  # bo32[i + 1] couples rows i and i + 1
    ho = np.zeros(nr + 1)
    ho[1:nr] = np.asarray(tab.hoff, np.float64)
    hd = np.asarray(tab.hd, np.float64).reshape(nl, nr)
    exact = tau64 * (hd + (ho[:-1] + ho[1:])[None, :])
    return exact - (bd32 + (bo32[:-1] + bo32[1:])[None, :])


def _sh_host_arrays(tab: ShTables, precision) -> dict:
    """The host arrays a spherical-harmonic simulation uploads (None where
    absent), by attribute name, in their device dtype."""
    precision = Precision(precision)
    f64, f32 = np.float64, np.float32
    c128 = precision == Precision.C128
    x = precision == Precision.C64X
    a = {}
    # psi goes up as its nonzero l rows only (an initial state is usually a few
    # l components: hydrogen 1s has one), complex128; the device zeroes the
    # other rows and, for the complex64 forms, splits these into g and (c64x)
    # its packed residual g_lo (ion_psi_split_c128)
    rows = sh_nonzero_rows(tab)
    if not rows.size:
        a["g_in"] = np.zeros((1, tab.n_r), np.complex128)
    elif tab.g0_row_data is not None:
        a["g_in"] = np.ascontiguousarray(tab.g0_row_data, dtype=np.complex128).reshape(rows.size, tab.n_r)
    else:
        a["g_in"] = np.ascontiguousarray(np.asarray(tab.g0, dtype=np.complex128).reshape(tab.n_l, tab.n_r)[rows])
    a["d_hd"] = np.asarray(tab.hd, f64) if c128 else None
    # c64x: the FP64 per-r diagonal tables the device forms the row-sum
    # remainders from (ion_sh_row_lo_c64)
    a["d_kinv64"] = np.asarray(tab.kinv, f64) if x else None
    a["d_cent64"] = np.asarray(tab.cent, f64) if x else None
    a["d_hoff"] = np.asarray(tab.hoff, f64)  # the complex64 forms' row-sum remainders read it too
    # the complex64 rotation pass reads the FP32 copies below
    a["d_rq"] = np.asarray(tab.rq, f64) if c128 else None
    a["d_cl"] = np.asarray(tab.cl, f64) if c128 else None
    a["d_mask"] = np.asarray(tab.mask, f64) if (tab.mask is not None and c128) else None
    a["d_tau"] = np.asarray(tab.tau, f64)
    a["d_ef"] = np.asarray(tab.efield, f64)
    # per-r FP32 tables zero-padded to a multiple of 16 entries: the radial
    # solve reads a chunk of 8 or 16 rows with 16-byte vector loads
    a["d_kinv32"] = _pad16(tab.kinv).astype(f32)
    a["d_cent32"] = _pad16(tab.cent).astype(f32)
    a["d_hoff32"] = _pad16(tab.hoff).astype(f32)
    a["d_rq32"] = np.asarray(tab.rq, f32)
    a["d_cl32"] = np.asarray(tab.cl, f32)
    a["d_mask32"] = np.asarray(tab.mask, f32) if tab.mask is not None else None
    vel = int(tab.gauge) == nat.ION_GAUGE_VELOCITY
    a["d_h2r"] = np.asarray(tab.h2r, f64) if vel else None
    a["d_h2r32"] = np.asarray(tab.h2r, f32) if vel else None
    n_states = len(tab.state_l)
    a["d_state_l"] = np.asarray(tab.state_l, dtype=np.int32).reshape(-1)
    if not n_states:
        a["d_state_g"] = np.zeros(2)
    elif sh_states_real(tab):  # real states: the kernels read one double a point
        a["d_state_g"] = np.ascontiguousarray(tab.state_g, dtype=np.float64).reshape(-1)
    else:
        a["d_state_g"] = np.asarray(tab.state_g, dtype=np.complex128).reshape(n_states, tab.n_r).view(
            np.float64).reshape(-1)
    return a


def sh_states_real(tab: ShTables) -> bool:
    """Whether the tables hold the test states as real values (float64)."""
    return np.asarray(tab.state_g).dtype == np.float64


def _sh_device_sizes(tab: ShTables):
    """(n_data, n_states, n_tiles) of a simulation's device-only buffers."""
    n_states = len(tab.state_l)
    return n_data_slots(int(tab.t_final), int(tab.store_every)), n_states, (tab.n_r + SH_ROT_ROWS - 1) // SH_ROT_ROWS


class _Arena:
    """Arrays of one dtype packed into one host buffer, uploaded with
    one copy; each array becomes a view of the device buffer.  Arrays added
    with ``align`` start on a 64-byte boundary (the first of each kind: the
    radial solve's float4 table loads need 16); the others follow the
    previous one directly, so a kind's arrays form one run that is packed with
    one copy.  The arrays of a kind keep the alignment their element needs
    because every array's byte size is a whole number of those elements (the
    FP32 tables the solve reads by float4 are padded to 64 bytes)."""

    def __init__(self, np_dtype):
        self.np_dtype = np.dtype(np_dtype)
        self.items = []  # (key, array, offset)
        self.placed = {}  # id(array) -> (array, offset): each array object once
        self.size = 0

    def add(self, key, arr, align=True):
        """Place ``arr``; the same array object added again shares its place."""
        if id(arr) in self.placed:
            self.items.append((key, arr, self.placed[id(arr)][1]))
            return
        if align:
            a = max(1, 64 // self.np_dtype.itemsize)
            self.size = (self.size + a - 1) // a * a
        self.items.append((key, arr, self.size))
        self.placed[id(arr)] = (arr, self.size)
        self.size += arr.size

    # Staged in a pageable host buffer, then one host-to-device copy.  On
    # GB300 (Grace host, NVLink-C2C) a copy from pageable memory that the host
    # has written runs at ~650 GB/s (229 MB in 1.3 ms), while page-locking a
    # fresh buffer of that size costs ~27 ms.  The packing runs in the
    # calling thread: for the thousands of arrays of a batch, 4 or 16 threads
    # took longer (23-28 ms against 21 ms for 229 MB).

    def runs(self):
        """(offset, [arrays]) of the placed arrays that follow one another."""
        out = []
        for arr, off in sorted(self.placed.values(), key=lambda x: x[1]):
            if out and out[-1][0] + out[-1][2] == off:
                out[-1][1].append(arr)
                out[-1][2] += arr.size
            else:
                out.append([off, [arr], arr.size])
        return [(off, arrs) for off, arrs, _ in out]

    def upload(self, tensors=()) -> dict:
        """Device views by key: torch views for the keys whose name is in
        ``tensors`` (keys are (index, name)), ``_DevSlice`` for the rest."""
        tdt = {np.dtype(np.float64): torch.float64, np.dtype(np.float32): torch.float32,
               np.dtype(np.int32): torch.int32, np.dtype(np.complex64): torch.complex64,
               np.dtype(np.complex128): torch.complex128}[self.np_dtype]
        n = max(self.size, 1)
        host = np.empty(n, dtype=self.np_dtype)
        for off, arrs in self.runs():  # one copy per run
            total = sum(a.size for a in arrs)
            np.concatenate([a.reshape(-1) for a in arrs], out=host[off:off + total])
        dev_buf = torch.empty(n, dtype=tdt, device=device())
        dev_buf.copy_(torch.from_numpy(host))
        return {key: (dev_buf[off:off + arr.size].view(arr.shape) if key[1] in tensors
                      else _DevSlice(dev_buf, off, arr.shape))
                for key, arr, off in self.items}


def sh_nonzero_rows(tab: "ShTables") -> np.ndarray:
    """The l rows of a simulation's initial psi that are not all zero."""
    if tab.g0_rows is not None:
        rows = np.asarray(tab.g0_rows, dtype=np.int64).reshape(-1)
        # the device writes these rows of psi: each must be a row of the mesh
        if rows.size and (rows.min() < 0 or rows.max() >= tab.n_l or np.unique(rows).size != rows.size):
            raise ValueError(f"initial-state rows {rows.tolist()} are not distinct rows of a mesh of {tab.n_l} l")
        return rows
    g0 = np.asarray(tab.g0).reshape(tab.n_l, tab.n_r)
    return np.flatnonzero(np.any(g0 != 0, axis=1)).astype(np.int64)


def _sh_state_buffers(total: int, precision, counts) -> List[dict]:
    """Device-only state of simulations, one dense buffer per kind sliced in
    order: g (complex128 or complex64), and for c64x g_lo (packed residual
    words) and d_row_lo (bf16 row-sum remainders).  Per simulation, by
    attribute."""
    precision = Precision(precision)
    out = [dict(g_lo=None, d_row_lo=None) for _ in counts]
    g = torch.empty(max(total, 1), dtype=complex_dtype(precision), device=device())
    lo = rl = None
    if precision == Precision.C64X:
        lo = torch.empty(max(total, 1), dtype=torch.int32, device=device())
        rl = torch.empty(max(total, 1), dtype=torch.int16, device=device())
    off = 0
    for i, n in enumerate(counts):
        out[i]["g"] = g[off:off + n]
        if lo is not None:
            out[i]["g_lo"] = lo[off:off + n]
            out[i]["d_row_lo"] = rl[off:off + n]
        off += n
    return out


def _sh_prepare(sims: List["ShDeviceSim"]):
    """Finish the upload of simulations on the device: psi zeroed and its
    uploaded rows put in place (complex64 forms: split into g and g_lo), then
    (c64x) the row-sum remainders of the radial step.  The uploaded rows are
    released."""
    todo = [s for s in sims if getattr(s, "g_in", None) is not None]
    bases = {}
    for s in todo:
        s.g = s.g.reshape(s.n_l, s.n_r)
        if s.g_lo is not None:
            s.g_lo = s.g_lo.reshape(s.n_l, s.n_r)
        for t in (s.g, s.g_lo):
            if t is not None:
                b = t._base if t._base is not None else t
                bases.setdefault(id(b), b)
    for b in bases.values():  # the state buffers are dense runs: one fill each
        b.zero_()
    # every uploaded row into place with one launch: a table of (source,
    # destination hi, destination lo, length) addresses
    table = []
    for s in todo:
        n = s.n_r
        src, hi = s.g_in.data_ptr(), s.g.data_ptr()
        lo = 0 if s.g_lo is None else s.g_lo.data_ptr()
        hs = s.g.element_size()
        for k, l in enumerate(s.g_rows):
            table.append((src + 16 * k * n, hi + hs * int(l) * n, lo + 4 * int(l) * n if lo else 0, n))
    if table:
        assert ctypes.sizeof(nat.PsiRow) == 32
        d_table = torch.from_numpy(np.array(table, dtype=np.int64)).to(device())
        c128 = todo[0].g.dtype == torch.complex128
        nat.call("ion_psi_split_rows_c128", len(table), d_table.data_ptr(), int(c128), stream_ptr())
    rows = [s for s in todo if getattr(s, "d_row_lo", None) is not None]
    if rows:
        nat.call("ion_sh_row_lo_c64", ctypes.byref(ShBatch(rows[0].precision, rows).plan), stream_ptr())
    if todo:
        torch.cuda.current_stream().synchronize()  # before the uploaded psi is released
    for s in todo:
        s.g_in = None


class ShDeviceSim:
    """Device buffers of one spherical-harmonic simulation.  ``arrays``: the
    device tensors by attribute name, when built together with others
    (``ShDeviceSim.bulk``); otherwise each host array is uploaded on its own."""

    def __init__(self, tab: ShTables, precision, arrays: Optional[dict] = None):
        self.precision = Precision(precision)
        self.tab = tab
        self.n_r, self.n_l = tab.n_r, tab.n_l
        self.t = int(tab.t0)
        self.t_final = int(tab.t_final)
        self.store_every = int(tab.store_every)
        self.gauge = int(tab.gauge)
        if arrays is None:
            host = _sh_host_arrays(tab, precision)
            self.h2d_bytes = sum(int(v.size) * np.dtype(v.dtype).itemsize for v in host.values() if v is not None)
            arrays = {k: (to_dev(v) if v is not None else None) for k, v in host.items()}
            arrays.update(_sh_state_buffers(tab.n_l * tab.n_r, self.precision, [tab.n_l * tab.n_r])[0])
            self.n_data, n_states, self.n_tiles = _sh_device_sizes(tab)
            arrays["d_norm"] = torch.full((self.n_data,), float("nan"), dtype=torch.float64, device=device())
            arrays["d_ip"] = torch.full((self.n_data * max(n_states, 1) * 2,), float("nan"), dtype=torch.float64,
                                        device=device())
            arrays["d_partials"] = torch.zeros(self.n_tiles * (1 + 2 * n_states), dtype=torch.float64,
                                               device=device())
        else:
            self.n_data, n_states, self.n_tiles = _sh_device_sizes(tab)
        for k, v in arrays.items():
            setattr(self, k, v)
        self.n_states = n_states
        self.g_rows = [int(l) for l in sh_nonzero_rows(tab)]
        self.d_spike_s = self.d_spike_t = self.d_edge = None
        if tab.hcross is not None:
            self._build_spikes()
        if self.g_in is not None and not getattr(self, "_deferred", False):
            _sh_prepare([self])

    def _build_spikes(self):
        """The coupled-line spikes s_l = A_l^-1 e_first and t_l = A_l^-1 e_last
        of every line (A_l = 1 + i tau H_l at the run's uniform tau), solved on
        the device by the batched Thomas solve, and the line-end scratch."""
        from . import cy

        if self.precision != Precision.C128:
            raise ValueError("coupled lines have a complex128 form only")
        L, n = self.n_l, self.n_r
        tau = float(self.tab.tau[min(self.t + 1, len(self.tab.tau) - 1)])
        diag = 1 + 1j * tau * np.asarray(self.tab.hd, dtype=np.float64)
        off = np.zeros(L * n - 1, dtype=np.complex128)
        for l in range(L):
            off[l * n: l * n + n - 1] = 1j * tau * np.asarray(self.tab.hoff, dtype=np.float64)
        d_off, d_diag = to_dev(off), to_dev(diag)
        e_first = np.zeros(L * n, dtype=np.complex128)
        e_first[::n] = 1.0
        e_last = np.zeros(L * n, dtype=np.complex128)
        e_last[n - 1::n] = 1.0
        self.d_spike_s = cy.tdma_batched_device(L, n, d_off, d_diag, d_off, to_dev(e_first))
        self.d_spike_t = cy.tdma_batched_device(L, n, d_off, d_diag, d_off, to_dev(e_last))
        self.d_edge = torch.zeros(4 * L, dtype=torch.complex128, device=device())

    @classmethod
    def bulk(cls, tables: List[ShTables], precision) -> List["ShDeviceSim"]:
        """Many simulations with one upload per dtype and one device
        buffer per kind of array."""
        arenas = {}
        # one after another: these are many small numpy calls, which a thread
        # pool only serialises on the GIL at a cost (8 workers: 0.2 s slower
        # for a 512-simulation sweep)
        per = [_sh_host_arrays(tab, precision) for tab in tables]
        # time-step tables that are equal (the same grid of times) are
        # uploaded once and shared
        by_key = {}
        for host in per:
            tau = host.get("d_tau")
            if tau is None or tau.size < 2:
                continue
            key = (tau.size, float(tau[1]), float(tau[-1]))
            for other in by_key.get(key, ()):
                if np.array_equal(other, tau):
                    host["d_tau"] = other
                    break
            else:
                by_key.setdefault(key, []).append(tau)
        # every simulation's uploaded psi rows first, then the tables
        order = ["g_in"] + [k for k in (per[0] if per else {}) if k != "g_in"]
        for k in order:
            first = True
            for i, host in enumerate(per):
                v = host.get(k)
                if v is not None:
                    arenas.setdefault(v.dtype, _Arena(v.dtype)).add((i, k), v, align=first)
                    first = False
        views = {}
        for ar in arenas.values():
            views.update(ar.upload(tensors=("g_in",)))
        # g, g_lo and the row remainders, each one dense run over the
        # simulations (psi = g + g_lo is formed over the whole run at once by
        # sh_psi_many)
        counts = [tab.n_l * tab.n_r for tab in tables]
        state = _sh_state_buffers(sum(counts), Precision(precision), counts)
        torch.cuda.current_stream().synchronize()  # the host sources are released below
        sizes = [_sh_device_sizes(tab) for tab in tables]
        n_norm = sum(nd for nd, _, _ in sizes)
        n_ip = sum(nd * max(ns, 1) * 2 for nd, ns, _ in sizes)
        n_part = sum(nt * (1 + 2 * ns) for _, ns, nt in sizes)
        d_norm = torch.full((max(n_norm, 1),), float("nan"), dtype=torch.float64, device=device())
        d_ip = torch.full((max(n_ip, 1),), float("nan"), dtype=torch.float64, device=device())
        d_part = torch.zeros(max(n_part, 1), dtype=torch.float64, device=device())
        sims, o_norm, o_ip, o_part = [], 0, 0, 0
        counted = set()  # a shared array's bytes count for the first simulation only
        for i, tab in enumerate(tables):
            nd, ns, nt = sizes[i]
            arrays = {k: views.get((i, k)) for k in per[i]}
            arrays.update(state[i])
            arrays["d_norm"] = _DevSlice(d_norm, o_norm, (nd,))
            arrays["d_ip"] = _DevSlice(d_ip, o_ip, (nd * max(ns, 1) * 2,))
            arrays["d_partials"] = _DevSlice(d_part, o_part, (nt * (1 + 2 * ns),))
            sim = cls.__new__(cls)
            sim._deferred = True  # prepared together below
            sim.__init__(tab, precision, arrays=arrays)
            sim.h2d_bytes = sum(int(v.size) * np.dtype(v.dtype).itemsize for v in per[i].values()
                                if v is not None and id(v) not in counted)
            counted.update(id(v) for v in per[i].values() if v is not None)
            sim._bulk = dict(norm=(d_norm, o_norm, nd), ip=(d_ip, o_ip, nd * max(ns, 1) * 2))
            o_norm += nd
            o_ip += nd * max(ns, 1) * 2
            o_part += nt * (1 + 2 * ns)
            sims.append(sim)
        _sh_prepare(sims)
        return sims


    def nbytes(self) -> int:
        tot = 0
        for v in vars(self).values():
            if isinstance(v, (torch.Tensor, _DevSlice)):
                tot += v.numel() * v.element_size()
        return tot

    def descriptor(self) -> nat.ShSim:
        d = nat.ShSim()
        d.g = ptr(self.g)
        d.n_r, d.n_l = self.n_r, self.n_l
        d.t, d.t_final, d.store_every = self.t, self.t_final, self.store_every
        d.hd, d.hoff, d.rq, d.cl = ptr(self.d_hd), ptr(self.d_hoff), ptr(self.d_rq), ptr(self.d_cl)
        d.mask, d.tau, d.efield = ptr(self.d_mask), ptr(self.d_tau), ptr(self.d_ef)
        d.kinv32, d.cent32, d.hoff32 = ptr(self.d_kinv32), ptr(self.d_cent32), ptr(self.d_hoff32)
        d.rq32, d.cl32, d.mask32 = ptr(self.d_rq32), ptr(self.d_cl32), ptr(self.d_mask32)
        d.corr0_32 = float(self.tab.corr0)
        d.n_states = self.n_states
        d.state_l, d.state_g = ptr(self.d_state_l), ptr(self.d_state_g)
        d.weight = float(self.tab.weight)
        d.out_norm, d.out_ip, d.partials = ptr(self.d_norm), ptr(self.d_ip), ptr(self.d_partials)
        d.n_tiles = self.n_tiles
        d.g_lo = ptr(self.g_lo)
        d.gauge = self.gauge
        d.h2r, d.h2r32 = ptr(self.d_h2r), ptr(self.d_h2r32)
        d.row_lo = ptr(self.d_row_lo)
        d.kinv, d.cent, d.corr0 = ptr(self.d_kinv64), ptr(self.d_cent64), float(self.tab.corr0)
        d.spike_s, d.spike_t, d.edge = ptr(self.d_spike_s), ptr(self.d_spike_t), ptr(self.d_edge)
        d.hcross = float(self.tab.hcross or 0.0)
        d.state_real = int(self.n_states > 0 and sh_states_real(self.tab))
        return d

    def data(self):
        """(norm[n_data], inner_products[n_states, n_data]) on the host."""
        norm = _tensor(self.d_norm).cpu().numpy()
        ip = _tensor(self.d_ip).cpu().numpy()[: self.n_data * self.n_states * 2].view(np.complex128)
        return norm, ip.reshape(self.n_data, self.n_states).T.copy()

    def psi_host(self) -> np.ndarray:
        g = self.g.cpu().numpy().astype(np.complex128)
        if self.g_lo is not None:
            g = g + lo_unpack(self.g_lo.cpu().numpy())
        return g


def _in_threads(fn, items, workers: int = 16):
    """``fn`` over ``items`` on up to ``workers`` threads (numpy copies and
    fills release the GIL); in the calling thread for one item."""
    items = list(items)
    k = max(1, min(workers, len(items), os.cpu_count() or 1))
    if k == 1:
        for it in items:
            fn(it)
        return
    with concurrent.futures.ThreadPoolExecutor(max_workers=k) as pool:
        list(pool.map(fn, items))


def _host_copy(t: torch.Tensor) -> np.ndarray:
    """One device-to-host copy into pageable memory whose pages the host
    touches first, with several threads for large buffers.  On GB300 the copy
    then runs at ~190 GB/s (837 MB: 4.5 ms after 8-17 ms of touching), where a
    copy into untouched pages runs at ~29 GB/s and a fresh page-locked buffer
    of that size costs ~75 ms to allocate."""
    out = np.empty(tuple(t.shape), dtype=torch.empty(0, dtype=t.dtype).numpy().dtype)
    flat = out.reshape(-1)
    if out.nbytes >= (16 << 20):
        k = 16
        c = (flat.size + k - 1) // k
        _in_threads(lambda i: flat[i * c:(i + 1) * c].fill(0), range(k), k)
    torch.from_numpy(out).copy_(t)
    return out


def sh_data_many(sims: List["ShDeviceSim"]):
    """(norm, inner_products) of every simulation: with one copy per buffer
    when they were built together (``ShDeviceSim.bulk``), else one by one."""
    if not sims or not all(hasattr(s, "_bulk") for s in sims) or \
            len({id(s._bulk["norm"][0]) for s in sims}) != 1:
        return [s.data() for s in sims]
    norm_all = _host_copy(sims[0]._bulk["norm"][0])
    ip_all = _host_copy(sims[0]._bulk["ip"][0])
    out = []
    for s in sims:
        _, on, nn = s._bulk["norm"]
        _, oi, ni = s._bulk["ip"]
        ip = ip_all[oi:oi + ni][: s.n_data * s.n_states * 2].view(np.complex128)
        out.append((norm_all[on:on + nn].copy(), ip.reshape(s.n_data, s.n_states).T.copy()))
    return out


def _run_of(ts: List[torch.Tensor]):
    """(base, first offset, end offset) when the tensors are contiguous views
    of one buffer in increasing order, else None."""
    if not ts or any(t._base is None or not t.is_contiguous() for t in ts):
        return None
    base = ts[0]._base
    offs = [t.storage_offset() for t in ts]
    if any(t._base is not base for t in ts) or any(b < a for a, b in zip(offs, offs[1:])):
        return None
    return base, offs[0], offs[-1] + ts[-1].numel()


def sh_psi_many(sims: List["ShDeviceSim"]) -> List[np.ndarray]:
    """psi (g + g_lo) of every simulation, complex128.  When the g of all
    simulations are one run of a complex64 buffer, and their g_lo another run
    with the same layout (``ShDeviceSim.bulk``), psi is formed on the device
    over the whole run (ion_psi_to_c128) and read back with one copy; else
    one copy per storage buffer and the sum on the host."""
    gs = [s.g for s in sims]
    los = [s.g_lo for s in sims]
    rg = _run_of(gs)
    has_lo = all(t is not None for t in los)
    rl = _run_of(los) if has_lo else None
    # the residual words of the run laid out point for point like g
    if rg is not None and rg[0].dtype == torch.complex64 and (
            not any(t is not None for t in los) or
            (rl is not None and rg[2] - rg[1] == rl[2] - rl[1] and
             all(b.storage_offset() - rl[1] == a.storage_offset() - rg[1] for a, b in zip(gs, los)))):
        base, g0, g1 = rg
        flat = base.reshape(-1)
        psi = torch.empty(g1 - g0, dtype=torch.complex128, device=base.device)
        lo = rl[0].reshape(-1)[rl[1]:rl[2]] if rl is not None else None
        nat.call("ion_psi_to_c128", g1 - g0, ptr(flat[g0:g1]), ptr(lo), ptr(psi), stream_ptr())
        host = _host_copy(psi)
        return [host[g.storage_offset() - g0:g.storage_offset() - g0 + g.numel()].reshape(tuple(g.shape))
                for g in gs]
    bases = {}
    for s in sims:
        for t in (s.g, s.g_lo):
            if t is not None:
                b = t._base if t._base is not None else t
                bases.setdefault(id(b), b)
    host = {k: _host_copy(b).reshape(-1) for k, b in bases.items()}

    def view(t):
        b = t._base if t._base is not None else t
        off = t.storage_offset() - b.storage_offset()
        return host[id(b)][off:off + t.numel()].reshape(tuple(t.shape))

    def one(s):
        g = view(s.g).astype(np.complex128)
        if s.g_lo is not None:
            g += lo_unpack(view(s.g_lo))
        return g

    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as pool:  # numpy work outside the GIL
        return list(pool.map(one, sims))


class ShBatch:
    """Many spherical-harmonic simulations advanced together."""

    def __init__(self, precision, sims: Optional[List[ShDeviceSim]] = None, cn_rows: int = 0,
                 rot_rows: int = SH_ROT_ROWS, bucket_rows=None):
        self.precision = Precision(precision)
        self.sims: List[ShDeviceSim] = list(sims or [])
        self.cn_rows = int(cn_rows)
        # rows per thread of each radial bucket (largest lines first; 0 or
        # missing: cn_rows); a bucket's CTA is sized for its longest line at
        # its own rows
        self.bucket_rows = tuple(int(r) for r in (bucket_rows or ()))
        self.rot_rows = int(rot_rows)
        if self.rot_rows != SH_ROT_ROWS:
            raise ValueError("row tiles of the rotation pass are fixed by the partial-sum layout")
        self._plan = None
        self._keep = None

    def add(self, sim: ShDeviceSim):
        self.sims.append(sim)
        self._plan = None

    def remove(self, sim: ShDeviceSim):
        self.sims.remove(sim)
        self._plan = None

    def _build_plan(self):
        sims = self.sims
        descs = (nat.ShSim * max(len(sims), 1))()
        for i, s in enumerate(sims):
            descs[i] = s.descriptor()
        raw = np.frombuffer(bytes(descs), dtype=np.uint8).copy()
        d_descs = to_dev(raw)
        # radial items grouped in buckets of equal CTA size (largest first);
        # each bucket is one launch whose blocks have exactly the threads its
        # lines need
        rows = self.cn_rows or sh_default_rows(self.precision, max([s.n_r for s in sims] + [2]))
        bsize = sh_bucket_sizes([s.n_r for s in sims], self.precision, rows)
        n_r = np.array([s.n_r for s in sims], dtype=np.int64)
        n_l = np.array([s.n_l for s in sims], dtype=np.int64)
        n_t = np.array([s.n_tiles for s in sims], dtype=np.int64)

        def items(counts):
            # (simulation, index) for every index below each count, in order
            sim = np.repeat(np.arange(len(counts), dtype=np.int64), counts)
            first = np.repeat(np.cumsum(counts) - counts, counts)
            return sim, np.arange(sim.size, dtype=np.int64) - first

        # stable sorts: lines by CTA size, then n_r, descending; tiles by n_l
        cs, cl = items(n_l)
        order = np.lexsort((-n_r[cs], -bsize[cs]))
        cs, cl = cs[order], cl[order]
        rs, rk = items(n_t)
        order = np.argsort(-n_l[rs], kind="stable")
        rs, rk = rs[order], rk[order]
        cn = np.stack([cs, cl], axis=1).astype(np.int32) if cs.size else np.zeros((1, 2), np.int32)
        rot = np.stack([rs, rk], axis=1).astype(np.int32) if rs.size else np.zeros((1, 2), np.int32)
        d_cn = to_dev(cn.reshape(-1))
        d_rot = to_dev(rot.reshape(-1))
        plan = nat.ShPlan()
        plan.sims = ptr(d_descs)
        plan.n_sims = len(sims)
        plan.max_n_l = max([s.n_l for s in sims] + [1])
        plan.max_n_r = max([s.n_r for s in sims] + [2])
        plan.flags = nat.ION_SH_REFINE if any(s.g_lo is not None for s in sims) else 0
        if any(getattr(s, "d_spike_s", None) is not None for s in sims):
            plan.flags |= nat.ION_SH_COUPLED
        n_vel = sum(1 for s in sims if s.gauge == nat.ION_GAUGE_VELOCITY)
        if n_vel:
            plan.flags |= nat.ION_SH_VELOCITY | (nat.ION_SH_ONLY_VELOCITY if n_vel == len(sims) else 0)
        plan.cn_items = ptr(d_cn)
        plan.n_cn_items = int(cs.size)
        plan.cn_threads = _round32(max([sh_line_threads(s.n_r, self.precision, rows) for s in sims] + [1]))
        plan.rot_items = ptr(d_rot)
        plan.n_rot_items = int(rs.size)
        plan.rot_rows = self.rot_rows
        plan.cn_rows = rows
        bs_sorted = bsize[cs]
        starts = np.concatenate([[0], np.nonzero(np.diff(bs_sorted))[0] + 1]) if cs.size else np.zeros(0, np.int64)
        threads = [int(bs_sorted[k]) for k in starts]
        ends = [int(k) for k in starts[1:]] + ([int(cs.size)] if cs.size else [])
        plan.cn_threads = max(threads + [32])
        plan.n_cn_buckets = len(threads)
        nr_sorted = n_r[cs]
        for b, (e, th) in enumerate(zip(ends, threads)):
            plan.cn_bucket_end[b] = e
            plan.cn_bucket_threads[b] = th
            br = self.bucket_rows[b] if b < len(self.bucket_rows) else 0
            if br and br != rows:
                th_b = _round32(sh_line_threads(int(nr_sorted[starts[b]]), self.precision, br))
                if br not in SH_ROWS_CHOICES[self.precision] or th_b > sh_max_line_threads(self.precision, br):
                    raise ValueError(f"bucket {b}: {br} rows per thread cannot hold its lines")
                plan.cn_bucket_threads[b] = th_b
                plan.cn_bucket_rows[b] = br
        self._plan = plan
        self._keep = (d_descs, d_cn, d_rot)

    @property
    def plan(self):
        if self._plan is None:
            self._build_plan()
        return self._plan

    def _fn(self, base):
        return base + ("_c128" if self.precision == Precision.C128 else "_c64")

    def run(self, n_steps: int):
        if n_steps <= 0 or not self.sims:
            return
        nat.call(self._fn("ion_sh_split_run"), ctypes.byref(self.plan), int(n_steps), stream_ptr())
        for s in self.sims:
            s.t = min(s.t + int(n_steps), s.t_final)

    def reduce(self):
        if self.sims:
            nat.call(self._fn("ion_sh_reduce"), ctypes.byref(self.plan), stream_ptr())

    def invalidate(self):
        """Rebuild descriptors on the next call (after host-side changes)."""
        self._plan = None


# ==========================================================================
# line mesh
# ==========================================================================


@dataclasses.dataclass
class LineTables:
    n: int
    method: int  # nat.ION_LINE_ADI, ION_LINE_SPLIT or ION_LINE_FFT
    hd: np.ndarray
    hoff: np.ndarray
    zq: np.ndarray
    mask: Optional[np.ndarray]
    tau: np.ndarray
    efield: np.ndarray
    state_g: np.ndarray  # [n_states, n] complex128
    weight: float
    g0: np.ndarray
    t0: int
    t_final: int
    store_every: int
    vstat: Optional[np.ndarray] = None  # ION_LINE_FFT: static potential
    kin: Optional[np.ndarray] = None  # ION_LINE_FFT: kinetic energies in bit-reversed order
    twiddle: Optional[np.ndarray] = None  # ION_LINE_FFT: exp(-2 pi i m / n)
    gauge: int = 0  # ION_GAUGE_VELOCITY: efield holds A(times[t]); vcoef = hbar (q/m) / (2 dz)
    vcoef: float = 0.0


def line_rows(precision) -> int:
    """Rows per thread of the line kernels (8 for complex128 and the residual
    form, 16 for complex64)."""
    return 16 if Precision(precision) == Precision.C64 else 8


def line_threads(n: int, precision) -> int:
    maxm = line_rows(precision)
    return (n + maxm - 1) // maxm  # the line is padded to whole chunks


LINE_MAX_CLUSTER = 8


def line_cta_max_n(precision) -> int:
    """Longest line one CTA of the line kernel holds."""
    return int(nat.value("ion_line_max_n_" + Precision(precision).value))


# Fewest points a CTA of a spread line keeps (measured on GB300, 10 lines of
# 2048-16384 points): a complex128 step is bound by one SM's FP64 rate, so
# down to one warp of chunks (256 points) more CTAs shorten it, 4096 points
# from 150 to 49 us per step with 8.  A complex64 step gains little (c64x,
# 16384 points: 53 -> 43 us with 8 CTAs) and loses below 2048 points per CTA,
# where the cluster barriers cost more than the elimination they share out,
# while each CTA of the residual form holds most of an SM's shared memory
# that a served mix's spherical-harmonic batches would use: complex64 lines
# keep 4096 points per CTA (c64x: no spreading beyond what the length needs).
LINE_SPREAD_MIN_POINTS = {Precision.C128: 256, Precision.C64: 4096, Precision.C64X: 4096}
# A line batch spreads every line this far by default.  The cluster size of a
# line depends on its length and precision only, never on its batch-mates, so
# a line's results are the same whichever lines share its launches.
LINE_DEFAULT_SPREAD = 8


def line_cluster(n: int, precision, cta_max: Optional[int] = None, spread: int = 1) -> int:
    """CTAs (a thread-block cluster when > 1) that advance a line of n points:
    as many as its length needs, or up to ``spread`` (at most 8) while each
    CTA keeps LINE_SPREAD_MIN_POINTS.  Spreading a line over more SMs
    shortens a step at the price of cluster barriers, so it pays where SMs
    would otherwise idle, as in a served mix with few lines."""
    precision = Precision(precision)
    cta_max = line_cta_max_n(precision) if cta_max is None else cta_max
    need = max(1, -(-int(n) // int(cta_max)))
    fit = max(1, int(n) // LINE_SPREAD_MIN_POINTS[precision])
    return max(need, min(int(spread), fit, LINE_MAX_CLUSTER))


class LineDeviceSim:
    def __init__(self, tab: LineTables, precision):
        self.precision = Precision(precision)
        self.tab = tab
        self.n = tab.n
        self.t = int(tab.t0)
        self.t_final = int(tab.t_final)
        self.store_every = int(tab.store_every)
        f64, f32 = np.float64, np.float32
        g0 = np.asarray(tab.g0, dtype=np.complex128)
        self.g = to_dev(g0).to(complex_dtype(precision))
        self.g_lo = None
        if self.precision == Precision.C64X:  # psi = g + g_lo (packed)
            hi = g0.astype(np.complex64)
            self.g_lo = to_dev(lo_pack(g0 - hi.astype(np.complex128)))
        self.d_hd, self.d_hoff, self.d_zq = to_dev(tab.hd, f64), to_dev(tab.hoff, f64), to_dev(tab.zq, f64)
        self.d_mask = to_dev(tab.mask, f64) if tab.mask is not None else None
        self.d_tau, self.d_ef = to_dev(tab.tau, f64), to_dev(tab.efield, f64)
        self.d_hd32, self.d_hoff32, self.d_zq32 = to_dev(tab.hd, f32), to_dev(tab.hoff, f32), to_dev(tab.zq, f32)
        self.d_mask32 = to_dev(tab.mask, f32) if tab.mask is not None else None
        self.d_hd_lo32 = self.d_hoff_lo32 = None
        if self.precision == Precision.C64X:
            self.d_hd_lo32, self.d_hoff_lo32 = to_dev(_lo32(tab.hd)), to_dev(_lo32(tab.hoff))
        self.d_vstat = self.d_vstat32 = self.d_kin = self.d_twiddle = None
        if tab.method == nat.ION_LINE_FFT:
            self.d_vstat, self.d_vstat32 = to_dev(tab.vstat, f64), to_dev(tab.vstat, f32)
            self.d_kin = to_dev(tab.kin, f64)
            self.d_twiddle = to_dev(np.asarray(tab.twiddle, np.complex128)).to(complex_dtype(precision))
        sg = np.asarray(tab.state_g, dtype=np.complex128).reshape(-1, self.n)
        self.n_states = sg.shape[0]
        self.d_state_g = to_dev(sg.view(np.float64).reshape(-1)) if self.n_states else to_dev(np.zeros(2))
        self.n_data = n_data_slots(self.t_final, self.store_every)
        self.d_norm = torch.full((self.n_data,), float("nan"), dtype=torch.float64, device=device())
        self.d_ip = torch.full((self.n_data * max(self.n_states, 1) * 2,), float("nan"), dtype=torch.float64,
                               device=device())

    def nbytes(self) -> int:
        return sum(v.numel() * v.element_size() for v in vars(self).values() if isinstance(v, torch.Tensor))

    def descriptor(self) -> nat.LineSim:
        d = nat.LineSim()
        d.g = ptr(self.g)
        d.n, d.method = self.n, int(self.tab.method)
        d.t, d.t_final, d.store_every = self.t, self.t_final, self.store_every
        d.hd, d.hoff, d.zq, d.mask = ptr(self.d_hd), ptr(self.d_hoff), ptr(self.d_zq), ptr(self.d_mask)
        d.tau, d.efield = ptr(self.d_tau), ptr(self.d_ef)
        d.hd32, d.hoff32, d.zq32, d.mask32 = ptr(self.d_hd32), ptr(self.d_hoff32), ptr(self.d_zq32), ptr(self.d_mask32)
        d.n_states = self.n_states
        d.state_g = ptr(self.d_state_g)
        d.weight = float(self.tab.weight)
        d.out_norm, d.out_ip = ptr(self.d_norm), ptr(self.d_ip)
        d.vstat, d.kin, d.twiddle, d.vstat32 = ptr(self.d_vstat), ptr(self.d_kin), ptr(self.d_twiddle), ptr(self.d_vstat32)
        d.g_lo = ptr(self.g_lo)
        d.gauge, d.vcoef = int(self.tab.gauge), float(self.tab.vcoef)
        d.hd_lo32, d.hoff_lo32 = ptr(self.d_hd_lo32), ptr(self.d_hoff_lo32)
        return d

    def data(self):
        norm = self.d_norm.cpu().numpy()
        ip = self.d_ip.cpu().numpy()[: self.n_data * self.n_states * 2].view(np.complex128)
        return norm, ip.reshape(self.n_data, self.n_states).T.copy()

    def psi_host(self) -> np.ndarray:
        g = self.g.cpu().numpy().astype(np.complex128)
        if self.g_lo is not None:
            g = g + lo_unpack(self.g_lo.cpu().numpy())
        return g


class LineBatch:
    """Line simulations advanced together: one launch per cluster size (lines
    up to one CTA's capacity in one launch, longer ones in thread-block
    clusters of 2..8 CTAs), any mix of methods, sizes and step counts."""

    def __init__(self, precision, sims: Optional[List[LineDeviceSim]] = None, spread: int = LINE_DEFAULT_SPREAD):
        self.precision = Precision(precision)
        self.sims: List[LineDeviceSim] = list(sims or [])
        self.spread = int(spread)  # CTAs per line where the line is short enough (line_cluster)
        self._plans = None
        self._keep = None
        self._cta_max = None

    def add(self, sim):
        self.sims.append(sim)
        self._plans = None

    def remove(self, sim):
        self.sims.remove(sim)
        self._plans = None

    def invalidate(self):
        self._plans = None

    def _cluster_of(self, sim) -> int:
        if self._cta_max is None:
            self._cta_max = line_cta_max_n(self.precision)
        # the Fourier split-step and velocity-gauge lines run in one CTA
        # (cluster plans skip them)
        one_cta = sim.tab.method == nat.ION_LINE_FFT or sim.tab.gauge == nat.ION_GAUGE_VELOCITY
        spread = 1 if one_cta else self.spread
        return line_cluster(sim.n, self.precision, self._cta_max, spread)

    @property
    def plans(self):
        if self._plans is None:
            groups = {}
            for s in self.sims:
                groups.setdefault(self._cluster_of(s), []).append(s)
            plans, keep = [], []
            maxm = line_rows(self.precision)
            for c in sorted(groups):
                sims = groups[c]
                descs = (nat.LineSim * len(sims))()
                for i, s in enumerate(sims):
                    descs[i] = s.descriptor()
                d = to_dev(np.frombuffer(bytes(descs), dtype=np.uint8).copy())
                p = nat.LinePlan()
                p.sims = ptr(d)
                p.n_sims = len(sims)
                p.max_n = max(s.n for s in sims)
                p.threads = _round32(max(-(-s.n // (c * maxm)) for s in sims))
                p.cluster = c
                p.flags = nat.ION_LINE_RESIDUAL if self.precision == Precision.C64X else 0
                if any(s.tab.method == nat.ION_LINE_FFT for s in sims):
                    p.flags |= nat.ION_LINE_HAS_FFT
                plans.append(p)
                keep.append(d)
            self._plans = plans
            self._keep = keep
        return self._plans

    @property
    def plan(self):
        """The single plan of a batch whose lines all take the same cluster size."""
        plans = self.plans
        if len(plans) != 1:
            raise ValueError("batch spans several cluster sizes; use .plans")
        return plans[0]

    def _fn(self, base):
        return base + ("_c128" if self.precision == Precision.C128 else "_c64")

    def run(self, n_steps: int):
        if n_steps <= 0 or not self.sims:
            return
        fn = self._fn("ion_line_run")
        for p in self.plans:
            nat.call(fn, ctypes.byref(p), int(n_steps), stream_ptr())
        for s in self.sims:
            s.t = min(s.t + int(n_steps), s.t_final)

    def reduce(self):
        if self.sims:
            fn = self._fn("ion_line_reduce")
            for p in self.plans:
                nat.call(fn, ctypes.byref(p), stream_ptr())


# ==========================================================================
# batched symmetric tridiagonal eigenpairs (numeric eigenstate bases)
# ==========================================================================


def tridiagonal_eigenpairs(diags: np.ndarray, offs: np.ndarray, max_value: float, max_count: int):
    """All eigenpairs with eigenvalue below ``max_value`` (at most
    ``max_count`` per matrix, the smallest) of each real symmetric tridiagonal
    matrix (rows of ``diags`` [n_mat, n], ``offs`` [n_mat, n-1]), on the
    device: Sturm counts, bisection, inverse iteration.  Returns a list of
    (values ascending, vectors [k, n] of unit 2-norm) per matrix."""
    diags = np.ascontiguousarray(diags, dtype=np.float64)
    offs = np.ascontiguousarray(offs, dtype=np.float64)
    n_mat, n = diags.shape
    d_d, d_o = to_dev(diags.reshape(-1)), to_dev(offs.reshape(-1))
    d_x = to_dev(np.full(n_mat, float(max_value)))
    d_cnt = torch.zeros(n_mat, dtype=torch.int32, device=device())
    sp = stream_ptr()
    nat.call("ion_tridiag_count_below", n_mat, n, ptr(d_d), ptr(d_o), ptr(d_x), ptr(d_cnt), sp)
    counts = np.minimum(d_cnt.cpu().numpy(), int(max_count))
    req_mat = np.concatenate([np.full(c, m, np.int32) for m, c in enumerate(counts)] + [np.zeros(0, np.int32)])
    req_idx = np.concatenate([np.arange(c, dtype=np.int32) for c in counts] + [np.zeros(0, np.int32)])
    n_req = len(req_mat)
    out = [(np.zeros(0), np.zeros((0, n))) for _ in range(n_mat)]
    if n_req == 0:
        return out
    d_rm, d_ri = to_dev(req_mat), to_dev(req_idx)
    d_vals = torch.empty(n_req, dtype=torch.float64, device=device())
    nat.call("ion_tridiag_eigvals", n_mat, n, ptr(d_d), ptr(d_o), n_req, ptr(d_rm), ptr(d_ri), ptr(d_vals), sp)
    d_vecs = torch.empty(n_req * n, dtype=torch.float64, device=device())
    d_scr = torch.empty(int(nat.value("ion_tridiag_eig_scratch_doubles", n, n_req)), dtype=torch.float64,
                        device=device())
    nat.call("ion_tridiag_eigvecs", n_mat, n, ptr(d_d), ptr(d_o), n_req, ptr(d_rm), ptr(d_vals), ptr(d_vecs),
             ptr(d_scr), sp)
    vals = d_vals.cpu().numpy()
    vecs = d_vecs.cpu().numpy().reshape(n_req, n)
    start = 0
    for m, c in enumerate(counts):
        out[m] = (vals[start:start + c].copy(), vecs[start:start + c].copy())
        start += c
    return out


# ==========================================================================
# whole-mesh reductions
# ==========================================================================


class Reducer:
    """norm and inner products of a device psi with fixed device states."""

    def __init__(self, M: int, states_c128: np.ndarray, weight: float):
        self.M = int(M)
        st = np.asarray(states_c128, dtype=np.complex128).reshape(-1, self.M)
        self.n_states = st.shape[0]
        self.d_states = to_dev(st.view(np.float64).reshape(-1)) if self.n_states else None
        self.weight = float(weight)
        nbytes = nat.value("ion_reduce_scratch_bytes", self.M, self.n_states)
        self.d_part = torch.empty(max(nbytes // 8, 1), dtype=torch.float64, device=device())

    def __call__(self, g: torch.Tensor, out_norm: torch.Tensor, out_ip: Optional[torch.Tensor]):
        fn = "ion_reduce_c128" if g.dtype == torch.complex128 else "ion_reduce_c64"
        nat.call(fn, self.M, ptr(g), self.n_states, ptr(self.d_states), self.weight, ptr(out_norm),
                 ptr(out_ip), ptr(self.d_part), stream_ptr())
