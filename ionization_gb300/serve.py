"""Served form: continuous batching of simulation requests on one GPU.

The reference has no server: a parameter scan runs one simulation per
HTCondor job (ionization_scans/scan_utils.py:638-663).  Here requests (line or
spherical-harmonic simulations, complex64 or complex128) arrive over time and
share the GPU:

* one device batch per (mesh kind, precision), each on its own CUDA stream, so
  the FP64-bound complex128 groups run beside the bandwidth-bound complex64
  groups;
* every iteration advances each non-empty batch by one chunk of steps (one
  launch sequence covers all its simulations whatever their sizes; a
  simulation that reaches its last step inside a chunk is skipped by the
  kernels for the rest of it);
* between chunks, arrived requests are admitted first come first served while
  their device memory fits the HBM budget, and finished ones are retired: their
  data are copied to the host and their buffers freed;
* a chunk is ~10 ms of GPU work (32 steps of a spherical-harmonic batch, 256
  of a line batch) and at most three per batch are in flight, so admission
  and retirement follow the GPU closely; a batch whose queue is full does not
  hold up the others, a new request's host tables are built on worker
  threads and its buffers uploaded on a separate stream, and line batches run
  on a higher-priority stream.

A request's results do not depend on which other requests shared its
launches (per-simulation tables, solver chunking, tiles and reduction order),
and every simulation meets chunk boundaries at the same steps of its own run
(multiples of its kind's chunk length from its admission), so a request served in a
mix is bit-identical to the same request served alone with the same chunk
length.  complex128 results do not depend on the chunk length either (they
equal the plain mesh path); complex64 ones do in the last bit, because the
rotation pass carries a compensation word across a step boundary only inside
one chunk.
"""

import collections
import concurrent.futures
import dataclasses
import time
from typing import Dict, List, Optional

import numpy as np
import torch

from . import _device as dev
from . import workloads
from .core import Precision

DEFAULT_HBM_BUDGET = 150 * 10 ** 9


@dataclasses.dataclass
class Request:
    id: int
    arrival: float  # seconds after the start of the run
    kind: str  # "line" or "sh"
    precision: str  # "c64x", "c64" or "c128"
    steps: int
    points: int  # z points of a line, radial points of a spherical-harmonic mesh
    l_bound: int = 0
    E0: float = 0.05
    omega: float = 0.057
    cycles: int = 4
    cep: float = 0.0

    @property
    def mesh_points(self) -> int:
        return self.points * (self.l_bound if self.kind == "sh" else 1)

    def spec(self, precision: Optional[str] = None):
        prec = precision or self.precision
        if self.kind == "sh":
            return workloads.sh_spec(f"request_{self.id}", self.points, self.l_bound, self.E0, self.omega,
                                     self.cycles, self.cep, self.steps, precision=prec)
        if self.kind == "line":
            return workloads.line_softcore(f"request_{self.id}", self.points, self.E0, self.omega, self.cycles,
                                           self.cep, self.steps, precision=prec)
        raise ValueError(f"unknown request kind {self.kind!r}")


def poisson_requests(n_requests=100, rate=20.0, seed=20261204, **kw) -> List[Request]:
    return [Request(**p) for p in workloads.poisson_scan_parameters(n_requests, rate, seed, **kw)]


@dataclasses.dataclass
class Completion:
    request: Request
    admitted: float
    finished: float
    norm: np.ndarray  # data-time norms (t = 0 and the last step)
    inner_products: np.ndarray  # [n_states, n_data]
    psi: Optional[np.ndarray] = None

    @property
    def latency(self) -> float:
        return self.finished - self.request.arrival

    @property
    def ground_population(self) -> float:
        """|<initial state | psi>|^2 at the last step."""
        return float(np.abs(self.inner_products[0, -1]) ** 2)


def host_tables(req: Request, precision: Optional[str] = None):
    """FP64 coefficient tables of a request, built on the host (no device)."""
    spec = req.spec(precision)
    spec.host_only = True
    return spec.to_sim().mesh.tables


def device_bytes(req: Request, precision: Optional[str] = None) -> int:
    """Device memory a request holds while it runs (psi, coefficient and field
    tables, test states, data buffers)."""
    prec = Precision(precision or req.precision)
    c = {Precision.C64: 8, Precision.C64X: 12}.get(prec, 16)  # c64x: complex64 + packed residual
    n_t = req.steps + 1
    if req.kind == "sh":
        nr, nl, ns = req.points, req.l_bound, 15
        # FP64 and FP32 per-r tables; c64x adds the bf16 row-sum remainders
        return (nr * nl * c + (nr * nl * 8 if prec == Precision.C128 else 0)
                + (nr * nl * 2 if prec == Precision.C64X else 0) + nr * (7 * 8 + 6 * 4)
                + nl * 12 + 2 * 8 * n_t + ns * nr * 16 + (nr // 32 + 1) * (1 + 2 * ns) * 8 + 4096)
    n = req.points
    return n * c + n * (4 * 8 + 6 * 4) + 2 * 8 * n_t + n * 16 + 4096


class _Group:
    def __init__(self, kind: str, precision: Precision):
        self.kind = kind
        self.precision = precision
        # Line steps are short launches of a few CTAs each; on a stream of
        # their own priority the block scheduler places them as soon as SMs
        # free up, instead of behind the spherical-harmonic groups' whole-GPU
        # launches.
        self.stream = torch.cuda.Stream(priority=-1 if kind == "line" else 0)
        self.batch = dev.ShBatch(precision) if kind == "sh" else dev.LineBatch(precision)
        self.inflight = collections.deque()  # events of enqueued chunks


class Server:
    """Continuous-batching server for ``Request`` objects on the current GPU."""

    def __init__(self, hbm_budget: int = DEFAULT_HBM_BUDGET, chunk_steps: int = 32, keep_psi: bool = False,
                 line_chunk_steps: int = 256, max_inflight: int = 3, table_workers: int = 4):
        self.hbm_budget = int(hbm_budget)
        # steps per chunk: a line step is ~30-100 us, a spherical-harmonic
        # batch step ~0.1-1 ms, so both kinds queue ~10 ms of work per chunk
        self.chunk_steps = int(chunk_steps)
        self.line_chunk_steps = int(line_chunk_steps)
        self.max_inflight = int(max_inflight)
        self.table_workers = int(table_workers)
        self.keep_psi = keep_psi
        self.groups: Dict[tuple, _Group] = {}
        self._upload = None
        self.used_bytes = 0  # reserved: device_bytes() of every active request
        self.peak_bytes = 0
        self.allocated_bytes = 0  # what the active requests' buffers actually hold
        self.peak_allocated_bytes = 0
        self.peak_active = 0

    def _group(self, req: Request) -> _Group:
        key = (req.kind, Precision(req.precision))
        g = self.groups.get(key)
        if g is None:
            g = self.groups[key] = _Group(*key)
        return g

    def _admit(self, req: Request, tables):
        """Upload a request on the upload stream (so the copies do not wait
        behind the group's running chunks); the group's stream waits for it on
        the device before its next chunk."""
        g = self._group(req)
        if self._upload is None:
            self._upload = torch.cuda.Stream()
        with torch.cuda.stream(self._upload):
            if req.kind == "sh":
                dsim = dev.ShDeviceSim(tables, g.precision)
                first = dev.ShBatch(g.precision, [dsim])
            else:
                dsim = dev.LineDeviceSim(tables, g.precision)
                first = dev.LineBatch(g.precision, [dsim])
            first.reduce()  # data at t = 0
            ready = torch.cuda.Event()
            ready.record(self._upload)
        g.stream.wait_event(ready)
        g.batch.add(dsim)
        return g, dsim

    def run(self, requests: List[Request], realtime: bool = True) -> List[Completion]:
        """Serve ``requests`` (arrival times in seconds from the start; with
        ``realtime`` False every request is available at once) and return
        their completions in finishing order."""
        with concurrent.futures.ThreadPoolExecutor(max_workers=self.table_workers) as pool:
            return self._run(requests, realtime, pool)

    def _run(self, requests, realtime, pool) -> List[Completion]:
        pending = collections.deque(sorted(requests, key=lambda r: (r.arrival, r.id)))
        building = collections.deque()  # arrived, host tables being built (arrival order)
        waiting = collections.deque()  # host tables built
        active = {}  # id -> (req, group, dsim, admitted, bytes)
        retiring = []  # (event, id)
        done: List[Completion] = []
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731

        while pending or building or waiting or active or retiring:
            now = clock()
            # host tables are built on worker threads (numpy, mostly outside
            # the GIL), so this loop keeps feeding the GPU meanwhile
            while pending and (not realtime or pending[0].arrival <= now):
                req = pending.popleft()
                building.append((req, pool.submit(host_tables, req)))
            while building and building[0][1].done():
                req, fut = building.popleft()
                waiting.append((req, fut.result()))
            while waiting:
                req, tables = waiting[0]
                need = device_bytes(req)
                if active and self.used_bytes + need > self.hbm_budget:
                    break
                waiting.popleft()
                g, dsim = self._admit(req, tables)
                self.used_bytes += need
                self.allocated_bytes += dsim.nbytes()
                active[req.id] = (req, g, dsim, clock(), need)
            self.peak_bytes = max(self.peak_bytes, self.used_bytes)
            self.peak_allocated_bytes = max(self.peak_allocated_bytes, self.allocated_bytes)
            self.peak_active = max(self.peak_active, len(active))

            # a chunk for every group with unfinished simulations and room in
            # its queue (max_inflight chunks); a full group does not hold up
            # the others
            moved = False
            for g in self.groups.values():
                while g.inflight and g.inflight[0].query():
                    g.inflight.popleft()
                if len(g.inflight) >= self.max_inflight or not any(s.t < s.t_final for s in g.batch.sims):
                    continue
                moved = True
                with torch.cuda.stream(g.stream):
                    g.batch.run(self.line_chunk_steps if g.kind == "line" else self.chunk_steps)
                    ev = torch.cuda.Event()
                    ev.record(g.stream)
                g.inflight.append(ev)
                for rid, (req, gg, dsim, adm, nb) in list(active.items()):
                    if gg is g and dsim.t >= dsim.t_final and not getattr(dsim, "_retiring", False):
                        dsim._retiring = True
                        retiring.append((ev, rid))

            # retire simulations whose last chunk has completed
            still = []
            for ev, rid in retiring:
                if ev.query():
                    moved = True
                    req, g, dsim, adm, nb = active.pop(rid)
                    norm, ips = dsim.data()
                    psi = dsim.psi_host() if self.keep_psi else None
                    g.batch.remove(dsim)
                    self.used_bytes -= nb
                    self.allocated_bytes -= dsim.nbytes()
                    done.append(Completion(req, adm, clock(), norm, ips, psi))
                else:
                    still.append((ev, rid))
            retiring = still

            if not active and not waiting and not building and pending and realtime:
                time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.05)))
            elif not moved:
                time.sleep(0.0005)  # every queue is full: let the GPU catch up
        torch.cuda.synchronize()
        return done


def summarize(completions: List[Completion], makespan: float) -> dict:
    lat = np.array([c.latency for c in completions])
    pts = sum(c.request.mesh_points * c.request.steps for c in completions)
    by_kind = collections.defaultdict(list)
    for c in completions:
        by_kind[f"{c.request.kind}_{c.request.precision}"].append(c.latency)
    return {
        "requests": len(completions),
        "makespan_s": round(makespan, 3),
        "latency_p50_s": round(float(np.percentile(lat, 50)), 3) if len(lat) else None,
        "latency_p99_s": round(float(np.percentile(lat, 99)), 3) if len(lat) else None,
        "latency_by_kind": {k: {"n": len(v), "p50_s": round(float(np.percentile(v, 50)), 3),
                                "p99_s": round(float(np.percentile(v, 99)), 3)} for k, v in sorted(by_kind.items())},
        "point_steps_per_s": pts / makespan if makespan > 0 else None,
        "requests_per_s": len(completions) / makespan if makespan > 0 else None,
    }


def _main(argv=None):
    import argparse
    import json

    ap = argparse.ArgumentParser(prog="python -m ionization_gb300.serve")
    ap.add_argument("--requests", type=int, default=100)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--seed", type=int, default=20261204)
    ap.add_argument("--chunk", type=int, default=32)
    a = ap.parse_args(argv)
    reqs = poisson_requests(a.requests, a.rate, a.seed)
    server = Server(chunk_steps=a.chunk)
    t = time.perf_counter()
    done = server.run(reqs)
    out = summarize(done, time.perf_counter() - t)
    out["peak_active"] = server.peak_active
    out["peak_reserved_bytes"] = server.peak_bytes
    out["peak_allocated_bytes"] = server.peak_allocated_bytes
    print(json.dumps(out))


if __name__ == "__main__":
    _main()
