"""Batched form: many independent spherical-harmonic simulations per step.

The reference runs parameter scans as one simulation per HTCondor job
(ionization_scans/scan_utils.py:638-663).  Here every simulation of a scan
lives in one device batch: each step is one launch of each fused kernel over
all simulations (radial solve of every (simulation, l) line; rotation / mask /
reduction pass over every (simulation, row tile); time-index advance), whatever
their sizes, pulses and step counts.  Runs are captured into CUDA graphs of
``graph_steps`` steps so the host issues one graph launch per chunk.

The launch shape (rows per thread of the radial solve, graph chunk) comes
from ``autotune``, a project-written autotuner that times candidates on the
actual batch.
"""

import time
from typing import List, Optional

import numpy as np
import torch

from . import _device as dev
from . import _native as nat
from .core import Precision


def _host_tables(spec):
    spec.host_only = True
    try:
        sim = spec.to_sim()
        return sim.mesh.tables, sim
    finally:
        spec.host_only = False


def host_tables_many(specs):
    """The host tables of many specifications, one after another (a thread
    pool was measured slower: most of the per-specification work holds the
    GIL)."""
    return [_host_tables(spec)[0] for spec in specs]


class BatchedSphericalHarmonicSimulation:
    """Advance ``specs`` (SphericalHarmonicSpecification, split operator,
    length gauge) together on one GPU.

    ``precision`` overrides the specifications' precision ("c64" stores psi
    in complex64 with FP64 fields, coefficient tables and reductions)."""

    def __init__(self, specs, precision: Optional[str] = None, graph_steps: int = 64, use_graphs: bool = True,
                 cn_rows: int = 0, tables=None, bucket_rows=None):
        self.specs = list(specs)
        self.precision = Precision(precision or self.specs[0].precision)
        if tables is None:
            tables = host_tables_many(self.specs)
        self.tables = tables
        dsims = dev.ShDeviceSim.bulk(tables, self.precision)  # one upload per dtype
        self.sims = dsims
        self.batch = dev.ShBatch(self.precision, dsims, cn_rows=cn_rows, bucket_rows=bucket_rows)
        self.graph_steps = int(graph_steps)
        self.use_graphs = use_graphs
        self._graphs = {}
        self._cap_stream = None
        self._started = False
        self.mesh_points = np.array([s.n_r * s.n_l for s in dsims], dtype=np.int64)

    @property
    def total_mesh_points(self) -> int:
        return int(self.mesh_points.sum())

    @property
    def steps_remaining(self) -> int:
        return max(s.t_final - s.t for s in self.sims)

    def start(self):
        if not self._started:
            self.batch.reduce()
            self._started = True

    def _graph_for(self, n):
        g = self._graphs.get(n)
        if g is None:
            torch.cuda.synchronize()
            g = torch.cuda.CUDAGraph()
            s = self._capture_stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                with torch.cuda.graph(g, stream=s):
                    nat.call(self.batch._fn("ion_sh_split_run"), nat.ctypes.byref(self.batch.plan), int(n),
                             dev.stream_ptr())
            torch.cuda.current_stream().wait_stream(s)
            self._graphs[n] = g
        return g

    def _capture_stream(self):
        """The one stream every graph of this batch is captured on.  The
        library makes the side streams a radial solve's buckets fork onto
        once per caller stream and only outside capture, so the first plain
        step runs on this stream too."""
        if self._cap_stream is None:
            self._cap_stream = torch.cuda.Stream()
        return self._cap_stream

    def step(self, n_steps: int = 1):
        """Advance every unfinished simulation by up to ``n_steps``."""
        self.start()
        n_steps = int(min(n_steps, self.steps_remaining))
        if n_steps <= 0:
            return
        if not self.use_graphs:
            self.batch.run(n_steps)
            return
        # first use: one plain step on the capture stream, so every kernel
        # attribute is set and that stream's side streams exist
        if not self._graphs and n_steps > 0:
            cs = self._capture_stream()
            cs.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(cs):
                self.batch.run(1)
            torch.cuda.current_stream().wait_stream(cs)
            n_steps -= 1
        k = self.graph_steps
        while n_steps >= k:
            self._graph_for(k).replay()
            for s in self.sims:
                s.t = min(s.t + k, s.t_final)
            n_steps -= k
        if n_steps:
            self.batch.run(n_steps)

    def run(self):
        self.step(self.steps_remaining)

    def results(self) -> List[dict]:
        torch.cuda.synchronize()
        out = []
        for spec, s, (norm, ips) in zip(self.specs, self.sims, dev.sh_data_many(self.sims)):
            states = list(spec.test_states)
            ov = np.abs(ips) ** 2  # (n_states, n_data), one array operation
            bound = [k for k, st in enumerate(states) if st.bound]
            out.append(dict(
                name=spec.name,
                t=s.t,
                norm=norm,
                inner_products=dict(zip(states, ips)),
                initial_state_overlap=ov[states.index(spec.initial_state)],
                bound_state_overlap=ov[bound].sum(axis=0) if bound else np.zeros_like(norm),
            ))
        return out

    def psi(self, i) -> np.ndarray:
        return self.sims[i].psi_host()

    def psi_all(self) -> List[np.ndarray]:
        """psi of every simulation (complex128), read back together."""
        torch.cuda.synchronize()
        return dev.sh_psi_many(self.sims)


def _time_steps(specs, precision, tables, rows, gs, steps, bucket_rows=()):
    """ms per step of ``steps`` steps through the API's own path (CUDA-graph
    replay of ``gs`` steps), after a warm-up that captures the graph."""
    b = BatchedSphericalHarmonicSimulation(specs, precision=precision, graph_steps=gs, cn_rows=rows, tables=tables,
                                           bucket_rows=bucket_rows)
    b.step(1 + gs)  # warm-up and capture
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(steps, gs) // gs * gs
    e0.record()
    b.step(n)
    e1.record()
    torch.cuda.synchronize()
    del b
    return e0.elapsed_time(e1) / n


def _bucket_lines(precision, tables, rows):
    """The longest n_r of each radial bucket of the plan at ``rows`` (largest
    first): the buckets ShBatch forms, without building the batch."""
    bsize = dev.sh_bucket_sizes([t.n_r for t in tables], precision, rows)
    return [max(t.n_r for t, b in zip(tables, bsize) if b == th) for th in sorted(set(bsize.tolist()), reverse=True)]


def autotune(specs, precision="c64", graph_steps=(16, 32, 64), steps=32, tables=None, per_bucket=True):
    """Choose the launch shape of a batch by timing candidates on it, in three
    stages: rows per thread of the radial solve for every bucket (which sets
    the threads per radial system and so the CTA size of every bucket); then,
    bucket by bucket (largest lines first), each other row count that holds
    the bucket's lines, kept when the whole step gets faster by more than 1 %;
    then the CUDA-graph chunk length.  Each candidate runs through the API's
    graph replay and is timed with CUDA events on the launching stream after
    a warm-up.  Returns (best, timings): best = dict(rows=, bucket_rows=,
    graph_steps=), timings = {candidate label: ms per step}."""
    precision = Precision(precision)
    if tables is None:
        tables = host_tables_many(specs)
    gs_mid = sorted(graph_steps)[len(graph_steps) // 2]
    timings = {}

    def label(rows, gs, br):
        extra = "".join(f"_b{b}r{r}" for b, r in enumerate(br) if r)
        return f"rows{rows}_graph{gs}{extra}"

    def run(rows, gs, br=()):
        key = label(rows, gs, br)
        if key not in timings:
            timings[key] = _time_steps(specs, precision, tables, rows, gs, steps, br)
        return timings[key]

    choices = dev.SH_ROWS_CHOICES[precision]
    rows = min(choices, key=lambda r: run(r, gs_mid))
    chosen = []
    if per_bucket:
        longest = _bucket_lines(precision, tables, rows)
        chosen = [0] * len(longest)
        best_t = run(rows, gs_mid)
        for b, n_r in enumerate(longest):
            for r in choices:
                if r == rows or -(-n_r // r) > dev.sh_max_line_threads(precision, r):
                    continue
                cand = list(chosen)
                cand[b] = r
                t = run(rows, gs_mid, tuple(cand))
                if t < 0.99 * best_t:
                    best_t, chosen = t, cand
    br = tuple(chosen)
    gs = min(graph_steps, key=lambda g: run(rows, g, br))
    return dict(rows=rows, bucket_rows=br, graph_steps=gs), timings


def plan_shape(batch: "BatchedSphericalHarmonicSimulation") -> dict:
    """The chosen plan's launch shape: the radial solve's buckets (CTA
    threads, lines) and the rotation pass's tiles."""
    p = batch.batch.plan
    ends = [int(p.cn_bucket_end[b]) for b in range(p.n_cn_buckets)]
    starts = [0] + ends[:-1]
    return {"radial_buckets": [{"threads": int(p.cn_bucket_threads[b]), "lines": ends[b] - starts[b],
                                "rows_per_thread": int(p.cn_bucket_rows[b] or p.cn_rows)}
                               for b in range(p.n_cn_buckets)],
            "rows_per_thread": int(p.cn_rows), "rotation_tiles": int(p.n_rot_items)}


def _main(argv=None):
    """Run the first ``--sims`` simulations of the seeded uneven sweep for a
    few steps and print the time per step: a small, self-contained case of
    the batched kernels (``python -m ionization_gb300.batch --sims 200``)."""
    import argparse

    from . import workloads as wl

    ap = argparse.ArgumentParser(prog="python -m ionization_gb300.batch")
    ap.add_argument("--sims", type=int, default=200)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--precision", default="c64", choices=["c64", "c64x", "c128"])
    ap.add_argument("--rows", type=int, default=None, help="rows per thread of the radial solve")
    ap.add_argument("--graphs", action="store_true", help="capture the steps in CUDA graphs")
    a = ap.parse_args(argv)
    specs = wl.uneven_sh_sweep(512, steps=10000, precision=a.precision)[: a.sims]
    b = BatchedSphericalHarmonicSimulation(specs, precision=a.precision, use_graphs=a.graphs, cn_rows=a.rows or 0)
    b.step(a.warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.step(a.steps)
    e1.record()
    torch.cuda.synchronize()
    pts = b.total_mesh_points
    ms = e0.elapsed_time(e1) / max(a.steps, 1)
    print(f"{len(specs)} simulations, {pts} mesh points, {a.precision}: {ms:.4f} ms/step, "
          f"{pts / ms * 1e3:.4g} point-steps/s")


if __name__ == "__main__":
    _main()
