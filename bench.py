#!/usr/bin/env python
"""Benchmark: batched uneven spherical-harmonic sweep on one GB300.

Workload ``uneven_sh_sweep``: 512 spherical-harmonic split-operator
simulations (Nr 800-3200 at dr 0.125, l_max 20-80, seeded pulses), 52.3 M
mesh points.  The headline configuration is c64x: complex64 arithmetic with
FP64 fields, coefficients and reductions, psi stored as complex64 plus its
rounding residual as two bf16 (12 B a point, 628 MB, larger than L2) and
refined radial solves whose residual uses the FP64 Hamiltonian, which keeps
the final populations of every simulation within 1e-6 of complex128 (see
``accuracy``); plain complex64 is timed beside it (``c64_plain``).  A step
advances all 512 simulations by one time step: three kernel launches (radial
solve buckets, one per range of line lengths, the rotation/mask/reduction
pass and the time-index advance).

Prints one JSON line:
  value      mesh-point-steps/s over the timed steps, psi resident in HBM
  e2e        the same metric through the public API from host buffers
             (H2D of psi and tables, the steps, D2H of data and psi)
  roofline   the dominant kernel's algorithmic bytes / its CUDA-event time
             against the measured HBM copy bandwidth
  cpu_baseline  the oracle (CPU restatement of the reference, complex128)
             on a bounded sample of the same workload on the host cores
  plain_c128 the single-simulation complex128 drop-in path (Nr 2000, l < 41)
  accuracy   |P_ground - P_ground(c128)| and the same for the ionization
             probability over the full 10000 steps, for every simulation of
             the sweep, for complex64 and for complex64 with a stored residual
             (c64x): max, p99, median
  per_config the 4096-point line (Crank-Nicolson and Fourier split-step), the
             Nr 2000 x l < 41 spherical-harmonic mesh and the 2000 x 1000
             cylindrical mesh on their own shapes: throughput, each dominant
             kernel's CUDA-event time against the roofline, and the oracle on
             one host core
  serving    the served scan mix (Poisson arrivals, lines and SH meshes of
             mixed sizes and precisions): p50/p99 latency, throughput, and
             every complex64 request's population error against the same
             request run in complex128

``--impl reference`` times the CPU oracle (the reference's algorithm,
complex128) on the same workload with all host cores instead.
Multi-GPU (torchrun): replicas, each rank its own seeded sweep, no collective
on the data path (weak scaling).
"""

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "mesh-pt-steps/s on 1 GB300: batched c64 vs plain c128 @≤1e-6 pop err; p50/p99 lat"
UNIT = "mesh-pt-steps/s"
SEED = 20261203
N_SIMS = 512
SIM_STEPS = 10000
FALLBACK_HBM_GBS = 6800.0


# --------------------------------------------------------------------------
# CPU oracle workers (spawned processes; import numpy/scipy only)
# --------------------------------------------------------------------------

_W = {}


def _oracle_sim(p, dt=0.02):
    from oracle import mesh as om
    from oracle import physics as ph

    T = p["cycles"] * 2 * np.pi / p["omega"]
    pulse = ph.CosSquaredPulse(p["E0"], p["omega"], p["cycles"], float(np.mod(p["cep"] + np.pi * p["cycles"], 2 * np.pi)),
                               T / 2)
    nr = p["r_points"]
    r_bound = 0.125 * (nr - 1)
    r_max = r_bound + 0.0625
    mask = dict(inner_radius=r_max - 25.0, outer_radius=r_max, smoothness=8)
    ts = [(n, l) for n in range(1, 6) for l in range(n)]
    return om.SphericalHarmonicSplit(nr, r_bound, p["l_bound"], pulse, mask, ts, dt)


def _worker_init(params):
    os.environ["OMP_NUM_THREADS"] = "1"
    import oracle

    oracle.build()
    _W["sims"] = [_oracle_sim(p) for p in params]
    _W["t"] = 0.0


def _worker_step(_):
    t0 = time.perf_counter()
    _W["t"] += 0.02
    for s in _W["sims"]:
        s.evolve(0.02, _W["t"])
    return time.perf_counter() - t0, sum(s.M for s in _W["sims"])


def _worker_run(args):
    params, steps = args
    os.environ["OMP_NUM_THREADS"] = "1"
    import oracle

    oracle.build()
    sims = [_oracle_sim(p) for p in params]
    t0 = time.perf_counter()
    t = 0.0
    for _ in range(steps):
        t += 0.02
        for s in sims:
            s.evolve(0.02, t)
    return time.perf_counter() - t0, sum(s.M for s in sims) * steps


def cpu_cores():
    return max(1, min(os.cpu_count() or 1, 64))


def cpu_baseline_sample(params, cores, steps=10):
    """Oracle throughput on ``cores`` processes, one slice of sims each."""
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    chunks = [params[i::cores] for i in range(cores)]
    chunks = [c for c in chunks if c]
    t0 = time.perf_counter()
    with ctx.Pool(len(chunks)) as pool:
        res = pool.map(_worker_run, [(c, steps) for c in chunks])
    wall = time.perf_counter() - t0
    pts = sum(r[1] for r in res)
    busy = max(r[0] for r in res)
    return pts / busy, wall, pts


# --------------------------------------------------------------------------
# helpers
# --------------------------------------------------------------------------


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def profile_fp64():
    """FP64-pipe utilisation of each per-configuration dominant kernel from the
    committed ncu summary (fraction of the pipe's peak, per kernel)."""
    path = os.path.join(ROOT, "profiles", "fp64_pipe.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def profile_traffic():
    """DRAM bytes per mesh point of each kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------


HEADLINE = "c64x"  # complex64 arithmetic, residual-compensated state: meets the 1e-6 bound


def time_batch(specs, tables, precision, K, warmup, rows, gs, local_rank, barrier, bucket_rows=()):
    """K steps of the whole batch through the API's own path (CUDA-graph
    replays of ``gs`` steps, the remainder launched directly), timed with CUDA
    events on the launching stream and the clocks sampled meanwhile; then,
    outside the timed region, min(K, 20) steps phase by phase with events
    around each radial solve and rotation pass for the per-kernel times."""
    import torch

    from ionization_gb300 import batch as bm

    b = bm.BatchedSphericalHarmonicSimulation(specs, precision=precision, graph_steps=gs, cn_rows=rows,
                                              tables=tables, bucket_rows=bucket_rows)
    b.step(gs + max(warmup, 3))  # captures the graph
    torch.cuda.synchronize()
    plan = b.batch.plan
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with Clocks(local_rank) as clk:
        e0.record(stream)
        b.step(K)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    elapsed = e0.elapsed_time(e1)
    # launches of the timed steps: per run of n steps one rotation pass before
    # the first solve, then per step the radial buckets, the rotation pass and
    # the advance
    per_step = max(int(plan.n_cn_buckets), 1) + 2
    runs = [gs] * (K // gs) + ([K % gs] if K % gs else [])
    launches = sum(1 + per_step * n for n in runs)
    out = time_phases(plan, precision, min(K, 20), stream)
    out.update(elapsed_ms=elapsed, launches=launches, clocks=clk.summary(), shape=bm.plan_shape(b))
    del b
    torch.cuda.synchronize()
    return out


def time_phases(plan, precision, K, stream):
    """K steps of an SH plan through ion_sh_split_phase with CUDA events on the
    launching stream around each radial solve and rotation pass."""
    import torch

    from ionization_gb300 import _native as nat

    fn = "ion_sh_split_phase_c128" if precision == "c128" else "ion_sh_split_phase_c64"
    sp = stream.cuda_stream
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    e_cn = [(ev(), ev()) for _ in range(K)]
    e_rot = [ev() for _ in range(K)]
    e0, e1 = ev(), ev()
    torch.cuda.synchronize()
    e0.record(stream)
    nat.call(fn, nat.ctypes.byref(plan), 1, sp)  # rotations before the first solve
    for k in range(K):
        e_cn[k][0].record(stream)
        nat.call(fn, nat.ctypes.byref(plan), 2, sp)
        e_cn[k][1].record(stream)
        nat.call(fn, nat.ctypes.byref(plan), 4 if k + 1 < K else 3, sp)
        e_rot[k].record(stream)
        nat.call(fn, nat.ctypes.byref(plan), 5, sp)
    e1.record(stream)
    torch.cuda.synchronize()
    return dict(elapsed_ms=e0.elapsed_time(e1),
                cn_ms=float(np.mean([a.elapsed_time(c) for a, c in e_cn])),
                rot_ms=float(np.mean([e_cn[k][1].elapsed_time(e_rot[k]) for k in range(K)])),
                launches=1 + (max(int(plan.n_cn_buckets), 1) + 2) * K)


def run_ours(args, rank, world, local_rank):
    import torch

    import ionization_gb300 as ig
    from ionization_gb300 import batch as bm
    from ionization_gb300 import replicas
    from ionization_gb300 import workloads as wl

    torch.cuda.set_device(local_rank)
    ig.build()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    barrier = replicas.barrier

    # ---- the workload: this rank's seeded sweep (replicas, weak scaling) ----
    t_setup = time.perf_counter()
    specs = wl.uneven_sh_sweep(N_SIMS, seed=replicas.sweep_seed(SEED, rank), steps=SIM_STEPS, precision=HEADLINE)
    tables = bm.host_tables_many(specs)
    setup_host_s = time.perf_counter() - t_setup
    points = int(sum(t.n_r * t.n_l for t in tables))

    if args.rows:  # a fixed launch shape (e.g. for a profiler run, whose timings would mislead the autotuner)
        best, tune = dict(rows=args.rows, bucket_rows=(), graph_steps=32), {}
    else:
        best, tune = bm.autotune(specs, HEADLINE, graph_steps=(16, 32, 64), steps=32, tables=tables)
    best_rows, best_gs, best_br = best["rows"], best["graph_steps"], best["bucket_rows"]

    # ---- timed region: K steps of the headline configuration ----
    K = args.steps
    main = time_batch(specs, tables, HEADLINE, K, args.warmup, best_rows, best_gs, local_rank, barrier, best_br)
    elapsed_ms = replicas.max_over_ranks(main["elapsed_ms"])
    cn_ms, rot_ms, clk_summary, gpu_launches = main["cn_ms"], main["rot_ms"], main["clocks"], main["launches"]
    # plain complex64 (no stored residual): faster, above the 1e-6 bound
    K64 = min(K, 100)
    t64 = time_batch(specs, tables, "c64", K64, args.warmup, 16, best_gs, local_rank, barrier)
    t64_ms = replicas.max_over_ranks(t64["elapsed_ms"])

    value = world * points * K / (elapsed_ms / 1e3)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None

    peak, peak_kind = measured_peaks()
    state_bytes = 12  # complex64 psi + its residual as two bf16 per point
    alg_bytes = 2 * state_bytes * points  # the state read once and written once per kernel
    dominant, dom_ms = ("sh_cn_pipelined", cn_ms) if cn_ms >= rot_ms else ("sh_rot_kernel", rot_ms)
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    pt = profile_traffic()
    traffic = pt.get(dominant + "_c64x_bytes_per_point")
    step_traffic = pt.get("step_total_c64x_bytes_per_point")
    roofline = {
        "bound": "hbm",
        "kernel": dominant,
        "achieved": round(achieved, 1),
        "peak": peak,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": round(achieved / peak, 4),
        "traffic": None if traffic is None else int(traffic * points),
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one steady-state step of this "
                          "512-simulation sweep (profiles/sh_dram_traffic_c64_uneven.md), per launch",
        "step_traffic": None if step_traffic is None else int(step_traffic * points),
        "step_algorithmic_bytes": 2 * alg_bytes,
        "algorithmic_bytes": alg_bytes,
        "kernel_ms": {"sh_cn_pipelined": round(cn_ms, 4), "sh_rot_kernel": round(rot_ms, 4)},
        "frac_by_kernel": {"sh_cn_pipelined": round(alg_bytes / (cn_ms / 1e3) / 1e9 / peak, 4),
                           "sh_rot_kernel": round(alg_bytes / (rot_ms / 1e3) / 1e9 / peak, 4)},
        # with a complex64 state's algorithmic bytes, 8 B each way per sweep
        "bytes_alg_c64": {"bytes_per_point": 16,
                          "frac_by_kernel": {k: round(16 * points / (v / 1e3) / 1e9 / peak, 4)
                                             for k, v in (("sh_cn_pipelined", cn_ms), ("sh_rot_kernel", rot_ms))}},
    }
    c64_plain = {
        "dtype": "c64", "value": world * points * K64 / (t64_ms / 1e3), "unit": UNIT, "steps": K64,
        "ms_per_step": t64_ms / K64,
        "kernel_ms": {"sh_cn_pipelined": round(t64["cn_ms"], 4), "sh_rot_kernel": round(t64["rot_ms"], 4)},
        "frac_by_kernel": {k: round(16 * points / (v / 1e3) / 1e9 / peak, 4)
                           for k, v in (("sh_cn_pipelined", t64["cn_ms"]), ("sh_rot_kernel", t64["rot_ms"]))},
        "note": "complex64 state without the stored residual: above the 1e-6 population bound (see accuracy)",
    }

    # ---- e2e through the public API from host buffers ----
    e2e = run_e2e(args, specs, tables, best_rows, best_gs, points, HEADLINE, best_br, setup_host_s)

    # ---- plain complex128 drop-in path, single simulation ----
    plain = run_plain_c128(args)

    # ---- accuracy of every simulation of the sweep: c64 forms vs c128 over the full run ----
    acc = None if args.quick else run_accuracy(None if args.accuracy == "full" else (0, 37, 101, 163, 255, 300, 411,
                                                                                     500))

    # ---- the line, SH and cylindrical workloads on their own shapes ----
    per_config = None if args.no_per_config else run_per_config(args, measured_peaks()[0])

    # ---- the served form ----
    serving = None if args.no_serve else run_serving(args)

    # ---- CPU oracle on a bounded sample ----
    cpu = None
    if not args.no_cpu:
        cores = cpu_cores()
        params = wl.uneven_sh_parameters(N_SIMS, SEED)
        sample = params[: 2 * cores]
        rate, wall, pts = cpu_baseline_sample(sample, cores, steps=args.cpu_steps)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"first {len(sample)} simulations of the sweep x {args.cpu_steps} steps on {cores} "
                         f"processes (complex128 oracle), {wall:.1f} s wall"}

    clocks = clk_summary
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": max(args.warmup, 3),
        "ms_per_step": elapsed_ms / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64",
        "data": "synthetic",
        "config": {
            "workload": "uneven_sh_sweep: 512 spherical-harmonic sims, Nr 800-3200, l_max 20-80, split operator",
            "precision": "c64x: complex64 arithmetic, FP64 fields / tables / reductions, psi stored as complex64 "
                         "+ its rounding residual as two bf16 (12 B a point), refined radial solves whose "
                         "residual uses the FP64 Hamiltonian",
            "n_sims": N_SIMS,
            "mesh_points": points,
            "state_bytes": points * state_bytes,
            "l2": f"inputs larger than L2 (state {points * state_bytes / 1e6:.0f} MB)",
            "parallelism": f"replicas x{world}",
            "autotune": {"chosen": {"cn_rows_per_thread": best_rows, "bucket_rows": list(best_br),
                                    "graph_steps": best_gs},
                         "plan": main["shape"],
                         "ms_per_step": {k: round(v, 4) for k, v in tune.items()}},
            "timing": "CUDA-graph replay of the API (graph_steps per replay, remainder launched directly); "
                      "per-kernel times from a separate phase-by-phase run of min(K, 20) steps",
            "host_setup_s": round(setup_host_s, 2),
        },
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": gpu_launches,
        "clocks": clocks,
        "plain_c128": plain,
        "c64_plain": c64_plain,
        "accuracy": acc,
        "per_config": per_config,
        "serving": serving,
    }
    if plain and plain.get("value"):
        out["vs_plain_c128"] = round(value / world / plain["value"], 2)
    if dist is not None:
        dist.destroy_process_group()
    return out


def run_e2e(args, specs, tables, rows, gs, points, precision, bucket_rows=(), host_setup_s=None):
    """Public API from host buffers: build the batch (H2D of psi, tables and
    field tables), K steps, then read back every simulation's data and psi."""
    import torch

    from ionization_gb300 import batch as bm

    K = args.steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = bm.BatchedSphericalHarmonicSimulation(specs, precision=precision, graph_steps=gs, cn_rows=rows, tables=tables,
                                              bucket_rows=bucket_rows)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    b.step(K)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    res = b.results()
    psis = b.psi_all()  # g (+ its residual) to the host
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    split = {"upload_s": round(t1 - t0, 3), "steps_s": round(t2 - t1, 3), "readback_s": round(wall - (t2 - t0), 3)}
    h2d = sum(s.h2d_bytes for s in b.sims)  # psi (complex128, split on the device) and the tables
    d2h = sum(s.g.numel() * 16 for s in b.sims)  # psi read back as complex128 (ion_psi_to_c128)
    d2h += sum(r["norm"].nbytes + 16 * len(r["inner_products"]) * len(r["norm"]) for r in res)
    del b, psis
    out = {"value": points * K / wall, "unit": UNIT, "h2d_bytes_per_step": int(h2d / K),
           "d2h_bytes_per_step": int(d2h / K), "steps": K, "wall_s": round(wall, 3), **split}
    if host_setup_s is not None:
        # from the specifications: the host tables (built before the timed
        # region, once for every run of the bench) added to the wall
        out["host_setup_s"] = round(host_setup_s, 3)
        out["value_with_host_setup"] = points * K / (wall + host_setup_s)
    return out


def run_serving(args):
    """The served scan mix: Poisson arrivals (20/s, seeded), lines of
    2048-16384 points and SH meshes of Nr 1000-4000 x l_max 20-100,
    2000-50000 steps, 80 % complex64 arithmetic (residual form), continuous
    batching under a 150 GB budget.  Latency = arrival to results on the
    host.  Error: the complex64 requests with the least work rerun in
    complex128 (the path matched to the reference), |P_ground - P_ground(c128)|."""
    import torch

    from ionization_gb300 import serve

    reqs = serve.poisson_requests(args.serve_requests, rate=20.0, seed=20261204)
    server = serve.Server()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done = server.run(reqs)
    makespan = time.perf_counter() - t0
    out = serve.summarize(done, makespan)
    out.update(workload=f"poisson_scan_parameters({args.serve_requests}, rate 20/s, seed 20261204)",
               peak_active=server.peak_active, peak_reserved_bytes=server.peak_bytes,
               mix={k: sum(1 for r in reqs if (r.kind, r.precision) == k)
                    for k in {(r.kind, r.precision) for r in reqs}})
    out["mix"] = {f"{k[0]}_{k[1]}": v for k, v in out["mix"].items()}
    # every complex64 request again in complex128 (the path matched to the
    # reference), all of them at once through one server without arrival times
    by_id = {c.request.id: c for c in done}
    low = [r for r in reqs if r.precision != "c128"]
    t1 = time.perf_counter()
    refs = serve.Server().run([serve.Request(**{**r.__dict__, "precision": "c128", "arrival": 0.0}) for r in low],
                              realtime=False)
    ref_wall = time.perf_counter() - t1
    ref_by_id = {c.request.id: c for c in refs}
    errs = {r.id: abs(by_id[r.id].ground_population - ref_by_id[r.id].ground_population) for r in low}
    ev = np.array(list(errs.values())) if errs else np.zeros(0)
    worst = max(errs, key=errs.get) if errs else None
    out["c64x_vs_c128_ground_population_err"] = {
        "requests": len(errs), "of_complex64_requests": len(low),
        "max": float(ev.max()) if ev.size else None,
        "p99": float(np.percentile(ev, 99)) if ev.size else None,
        "median": float(np.median(ev)) if ev.size else None,
        "over_1e-6": int(np.sum(ev > 1e-6)),
        "worst": None if worst is None else {"id": worst, "kind": by_id[worst].request.kind,
                                             "mesh_points": by_id[worst].request.mesh_points,
                                             "steps": by_id[worst].request.steps, "err": errs[worst]},
        "by_kind_max": {k: float(max(v for i, v in errs.items() if by_id[i].request.kind == k))
                        for k in {by_id[i].request.kind for i in errs}},
        "complex128_rerun_wall_s": round(ref_wall, 1)}
    return out


def run_plain_c128(args):
    import torch

    from ionization_gb300 import workloads as wl

    steps = 400 if args.quick else 2000
    spec = wl.sh_hydrogen_2000x41(steps=steps + 10, precision="c128")
    sim = spec.to_sim()
    sim.run(max_steps=5)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.run(max_steps=steps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    M = sim.mesh.mesh_points
    return {"workload": "sh_hydrogen_2000x41 (Nr 2000, l < 41, split operator)", "dtype": "c128",
            "value": M * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps, "steps": steps}


def run_accuracy(subset=None):
    """Final ground-state population and ionization probability of every
    simulation of the sweep (or of ``subset``): the complex64 batches against
    the complex128 batch (itself matched to the reference to <= 1e-10 on the
    single-simulation workloads) over all 10000 steps."""
    import torch

    from ionization_gb300 import batch as bm
    from ionization_gb300 import workloads as wl

    out, wall = {}, {}
    for prec in ("c128", "c64", "c64x"):
        specs = wl.uneven_sh_sweep(N_SIMS, seed=SEED, steps=SIM_STEPS, precision=prec,
                                   subset=None if subset is None else list(subset))
        t0 = time.perf_counter()
        b = bm.BatchedSphericalHarmonicSimulation(specs, precision=prec)
        b.run()
        out[prec] = b.results()
        del b
        torch.cuda.synchronize()
        wall[prec] = round(time.perf_counter() - t0, 1)
    pg = lambda r: float(r["initial_state_overlap"][-1])  # noqa: E731
    pion = lambda r: 1.0 - float(r["bound_state_overlap"][-1])  # noqa: E731
    res = {"n_instances": len(out["c128"]), "steps": SIM_STEPS,
           "subset": "all" if subset is None else list(subset), "wall_s": wall,
           # the same whole runs (set-up, 10000 steps, data) of the batched
           # complex128 form against the c64x form
           "c64x_vs_c128_batch_wall": round(wall["c128"] / max(wall["c64x"], 1e-9), 1),
           "ground_population_c128": {"min": min(pg(c) for c in out["c128"]),
                                      "median": float(np.median([pg(c) for c in out["c128"]]))},
           "ionization_probability_c128": {"max": max(pion(c) for c in out["c128"]),
                                           "median": float(np.median([pion(c) for c in out["c128"]]))}}
    for prec in ("c64", "c64x"):
        dg = np.array([abs(pg(a) - pg(c)) for a, c in zip(out[prec], out["c128"])])
        di = np.array([abs(pion(a) - pion(c)) for a, c in zip(out[prec], out["c128"])])
        res[prec] = {"max_abs_err_ground_population": float(dg.max()),
                     "p99_abs_err_ground_population": float(np.percentile(dg, 99)),
                     "median_abs_err_ground_population": float(np.median(dg)),
                     "max_abs_err_ionization_probability": float(di.max()),
                     "p99_abs_err_ionization_probability": float(np.percentile(di, 99)),
                     "worst_instance": int(np.argmax(dg)),
                     "instances_over_1e-6": int(np.sum(dg > 1e-6))}
    return res


# --------------------------------------------------------------------------
# per-configuration lines: the line, spherical-harmonic and cylindrical
# workloads on their own shapes, each beside the oracle on one host core
# --------------------------------------------------------------------------

# algorithmic bytes per mesh-point-step: one read and one write of psi per
# unavoidable sweep (the line: one sweep; SH split and cylindrical ADI: two)
B_ALG = {("line", "c128"): 32, ("line", "c64"): 16, ("sh", "c128"): 64, ("sh", "c64"): 32,
         ("cyl", "c128"): 64, ("cyl", "c64"): 32}


def _cpu_config(name, steps):
    """One core, the oracle on one per-configuration workload: seconds per step."""
    os.environ["OMP_NUM_THREADS"] = "1"
    import oracle
    from oracle import mesh as om
    from oracle import physics as ph

    oracle.build()

    def pulse(E0, omega, cycles, phase):
        T = cycles * 2 * np.pi / omega
        return ph.CosSquaredPulse(E0, omega, cycles, float(np.mod(phase + np.pi * cycles, 2 * np.pi)), T / 2)

    if name.startswith("line"):
        method = "FourierSplitOperator" if "fft" in name else "AlternatingDirectionImplicit"
        st = om.LineLength(4096, 100.0, 1.0, float(np.sqrt(2)), pulse(0.05, 0.057, 4, 0.0),
                           dict(inner_radius=80.0, outer_radius=100.0, smoothness=8), method)
        dt = 0.05
    elif name.startswith("sh"):
        st = om.SphericalHarmonicSplit(2000, 0.125 * 1999, 41, pulse(0.05, 0.057, 6, 0.0),
                                       dict(inner_radius=0.125 * 1999 + 0.0625 - 25.0,
                                            outer_radius=0.125 * 1999 + 0.0625, smoothness=8),
                                       [(n, l) for n in range(1, 6) for l in range(n)], 0.02)
        dt = 0.02
    else:
        T = 4 * 2 * np.pi / 0.1
        st = om.CylindricalSliceADI(2000, 100.0, 1000, 100.0,
                                    ph.CosSquaredPulse(0.02, 0.1, 4, float(np.mod(4 * np.pi, 2 * np.pi)), T / 2),
                                    [(1, 0), (2, 0), (2, 1)])
        dt = 0.02
    M = int(np.prod(st.g.shape))
    st.evolve(dt, dt)  # warm-up (first-call costs)
    t0 = time.perf_counter()
    for k in range(steps):
        st.evolve(dt, (k + 2) * dt)
    return (time.perf_counter() - t0) / steps, M


def _events(n):
    import torch

    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def _per_config_entry(name, workload, dtype, kind, points, K, total_ms, kernels, peak, cpu, fp64=None, resident=None):
    """One entry: throughput, the dominant kernel's event time against the
    roofline with the algorithmic bytes of the mesh kind, and the CPU oracle."""
    dom = max(kernels, key=kernels.get)
    dom_ms = kernels[dom]
    b_alg = B_ALG[(kind, "c128" if dtype == "c128" else "c64")]
    # per step the dominant kernel moves (its share of the sweeps) x B_alg
    sweeps = 1 if kind == "line" else 2
    per_kernel_bytes = b_alg * points / sweeps if len(kernels) > 1 else b_alg * points
    achieved = per_kernel_bytes / (dom_ms / 1e3) / 1e9
    value = points * K / (total_ms / 1e3)
    out = {
        "workload": workload, "dtype": dtype, "value": value, "unit": UNIT, "steps": K,
        "ms_per_step": total_ms / K, "mesh_points": points,
        "kernel_ms_per_step": {k: round(v, 5) for k, v in kernels.items()},
        "roofline": {"bound": "fp64" if dtype == "c128" else "hbm", "kernel": dom,
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "algorithmic_bytes_per_point_step": b_alg,
                     "fp64_pipe_frac": None if fp64 is None else fp64.get(dom)},
    }
    if resident:
        out["roofline"]["note"] = resident
    if cpu is not None:
        sec, m = cpu
        out["cpu_baseline"] = {"value": m / sec, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"the oracle (complex128) on the same mesh, one process, "
                                         f"{sec * 1e3:.1f} ms per step"}
        out["vs_cpu_1core"] = round(value / (m / sec), 1)
    return out


def run_per_config(args, peak):
    import multiprocessing as mp

    import torch

    from ionization_gb300 import _native as nat
    from ionization_gb300 import mesh
    from ionization_gb300 import workloads as wl

    want = set(args.configs.split(",")) if args.configs else {"line_cn_4096", "line_fft_4096", "sh_2000x41",
                                                               "cyl_2000x1000"}
    cpu_jobs = {k: n for k, n in {"line_cn_4096": 200, "line_fft_4096": 200, "sh_2000x41": 6,
                                  "cyl_2000x1000": 2}.items() if k in want}
    cpu = {}
    pool = None
    if not args.no_cpu:  # the CPU legs run in spawned processes while the GPU legs run
        pool = mp.get_context("spawn").Pool(len(cpu_jobs))
        cpu_async = {k: pool.apply_async(_cpu_config, (k, n)) for k, n in cpu_jobs.items()}
    prof = profile_fp64()
    stream = torch.cuda.current_stream()
    out = {}

    def timed_run(spec, K, W=20):
        sim = spec.to_sim()
        sim.run(max_steps=W)
        torch.cuda.synchronize()
        e0, e1 = _events(2)
        e0.record(stream)
        sim.run(max_steps=K)
        e1.record(stream)
        torch.cuda.synchronize()
        return sim, e0.elapsed_time(e1)

    # cfg 1: the 4096-point soft-core line, Crank-Nicolson (ADI), 4000 steps; one
    # launch runs all its steps, so the kernel time is the run's time
    for prec in ("c128", "c64x") if "line_cn_4096" in want else ():
        K = 4000
        spec = wl.line_softcore_4096(steps=K + 20, precision=prec)
        sim, ms = timed_run(spec, K)
        kern = "line_cluster_kernel" if prec == "c128" else "line_res_kernel"
        out[f"line_cn_4096_{prec}"] = dict(
            name="line_cn_4096", workload="line_softcore_4096: 4096 points, ADI Crank-Nicolson, 4000 steps",
            dtype=prec, kind="line", points=4096, K=K, total_ms=ms, kernels={kern: ms / K},
            resident="psi (64 KB) stays in shared memory through the launch: not an HBM-bound run")
        del sim
    # the Fourier split-step on the same line
    for prec in ("c128", "c64") if "line_fft_4096" in want else ():
        K = 4000
        spec = wl.line_softcore("line_fft_4096", 4096, 0.05, 0.057, 4, 0.0, K + 20, precision=prec,
                                evolution_method=mesh.FourierSplitOperator())
        sim, ms = timed_run(spec, K)
        out[f"line_fft_4096_{prec}"] = dict(
            name="line_fft_4096", workload="4096-point soft-core line, Fourier split-step, 4000 steps",
            dtype=prec, kind="line", points=4096, K=K, total_ms=ms, kernels={"line_step_kernel": ms / K},
            resident="psi stays in shared memory through the launch: not an HBM-bound run")
        del sim
    if "sh_2000x41" in want:
        # cfg 2: Nr 2000 x l < 41, split operator, complex128 (the plain drop-in)
        K = 400
        spec = wl.sh_hydrogen_2000x41(steps=K + 40, precision="c128")
        sim = spec.to_sim()
        sim.run(max_steps=20)
        torch.cuda.synchronize()
        plan = sim.mesh._batch.plan
        t = time_phases(plan, "c128", K, stream)
        out["sh_2000x41_c128"] = dict(
            name="sh_2000x41", workload="sh_hydrogen_2000x41: Nr 2000, l < 41, split operator, complex128",
            dtype="c128", kind="sh", points=82000, K=K, total_ms=t["elapsed_ms"],
            kernels={"sh_cn_pipelined": t["cn_ms"], "sh_rot_kernel": t["rot_ms"]},
            resident="psi (1.3 MB) is L2-resident: not an HBM-bound run")
        del sim
    psi_cyl = {}
    for prec in ("c128", "c64") if "cyl_2000x1000" in want else ():
        # cfg 3: cylindrical slice 2000 x 1000, ADI, complex128 (and the FP32
        # sweeps of the complex64 form beside it); each pass timed
        K = 50
        spec = wl.cyl_hydrogen_2000x1000(steps=K + 10, precision=prec)
        sim = spec.to_sim()
        sim.run(max_steps=5)
        torch.cuda.synchronize()
        m = sim.mesh
        t0 = m._t
        ev = _events(3 * K)
        fn = "ion_cyl_adi_pass_" + prec
        for k in range(K):
            tn = t0 + k + 1
            ev[3 * k].record(stream)
            nat.call(fn, m._cm, m._g.data_ptr(), m._gtmp.data_ptr(), tn, nat.ION_ADI_PASS_STRIDED, 0,
                     stream.cuda_stream)
            ev[3 * k + 1].record(stream)
            nat.call(fn, m._cm, m._gtmp.data_ptr(), m._g.data_ptr(), tn, nat.ION_ADI_PASS_CONTIG, 1,
                     stream.cuda_stream)
            ev[3 * k + 2].record(stream)
        torch.cuda.synchronize()
        zp = float(np.mean([ev[3 * k].elapsed_time(ev[3 * k + 1]) for k in range(K)]))
        rp = float(np.mean([ev[3 * k + 1].elapsed_time(ev[3 * k + 2]) for k in range(K)]))
        total = ev[0].elapsed_time(ev[-1])
        psi_cyl[prec] = m.g
        out[f"cyl_2000x1000_{prec}"] = dict(
            name="cyl_2000x1000", workload=f"cyl_hydrogen_2000x1000: 2000 (z) x 1000 (rho), ADI, {prec}",
            dtype=prec, kind="cyl", points=2_000_000, K=K, total_ms=total,
            kernels={"cyl_zpass_kernel": zp, "cyl_rhopass_kernel": rp},
            resident=f"psi {2_000_000 * (16 if prec == 'c128' else 8) // 10**6} MB: within L2 (129 MB) "
                     "between the passes")
        del sim, m
    if len(psi_cyl) == 2:
        a, b = psi_cyl["c64"], psi_cyl["c128"]
        out["cyl_2000x1000_c64"]["psi_rel_l2_vs_c128"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    torch.cuda.synchronize()
    if pool is not None:
        for k, r in cpu_async.items():
            try:
                cpu[k] = r.get(timeout=600)
            except Exception as e:  # noqa: BLE001 - the CPU leg is reported, never a gate
                cpu[k] = None
                print(f"per-config CPU leg {k} failed: {e}", file=sys.stderr)
        pool.close()
        pool.join()
    res = {}
    for key, d in out.items():
        res[key] = _per_config_entry(d["name"], d["workload"], d["dtype"], d["kind"], d["points"], d["K"],
                                     d["total_ms"], d["kernels"], peak, cpu.get(d["name"]),
                                     prof.get(key), d.get("resident"))
        if "psi_rel_l2_vs_c128" in d:
            res[key]["psi_rel_l2_vs_c128"] = d["psi_rel_l2_vs_c128"]
    return res


# --------------------------------------------------------------------------
# reference arm: the CPU oracle on all host cores
# --------------------------------------------------------------------------


def run_reference(args, rank, world):
    if rank != 0:
        return None
    import multiprocessing as mp

    from ionization_gb300 import workloads as wl

    cores = cpu_cores()
    params = wl.uneven_sh_parameters(N_SIMS, SEED)
    # size the per-step sample so that warm-up + timed steps fit the budget
    budget_s = float(os.environ.get("ION_REF_BUDGET_S", "150"))
    probe_rate = 2.5e6 * cores  # pt-steps/s, refined after the first step
    per_step = budget_s / (args.steps + max(args.warmup, 3))
    n_sample = 0
    pts = 0
    for p in params:
        if pts + p["r_points"] * p["l_bound"] > probe_rate * per_step:
            break
        pts += p["r_points"] * p["l_bound"]
        n_sample += 1
    n_sample = max(n_sample, min(cores, len(params)))
    sample = params[:n_sample]
    ctx = mp.get_context("spawn")
    chunks = [c for c in (sample[i::cores] for i in range(cores)) if c]
    times = []
    pools = [ctx.Pool(1, initializer=_worker_init, initargs=(c,)) for c in chunks]
    try:
        for k in range(max(args.warmup, 3) + args.steps):
            t0 = time.perf_counter()
            rs = [pl.apply_async(_worker_step, (0,)) for pl in pools]
            res = [r.get() for r in rs]
            dt = time.perf_counter() - t0
            if k >= max(args.warmup, 3):
                times.append(dt)
        M = sum(r[1] for r in res)
    finally:
        for pl in pools:
            pl.terminate()
    total = float(np.sum(times))
    value = M * len(times) / total
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c128",
        "data": "synthetic",
        "config": {"workload": "uneven_sh_sweep: 512 spherical-harmonic sims, split operator", "n_sims": N_SIMS,
                   "sample_sims_per_step": n_sample, "sample_mesh_points": M},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": len(chunks), "kind": "port",
                         "sample": f"{n_sample} of {N_SIMS} simulations advanced one step per timed step, "
                                   f"{len(chunks)} processes (complex128 oracle restating the reference)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip the 10000-step accuracy run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle sample")
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--no-serve", action="store_true", help="skip the served-mix run")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--accuracy", default="full", choices=["full", "subset"],
                    help="accuracy over all 512 simulations (default) or a seeded subset of 8")
    ap.add_argument("--no-per-config", action="store_true", help="skip the per-configuration lines")
    ap.add_argument("--configs", default="", help="comma list of per-configuration workloads to run "
                    "(line_cn_4096, line_fft_4096, sh_2000x41, cyl_2000x1000; default all)")
    ap.add_argument("--only-per-config", action="store_true",
                    help="run only the per-configuration lines and print them (a profiling case)")
    ap.add_argument("--rows", type=int, default=0, choices=[0, 4, 8, 16],
                    help="rows per thread of the radial solve; 0 = autotune")
    args = ap.parse_args()

    from ionization_gb300 import replicas

    rank, world, local_rank = replicas.rank_world()
    if args.only_per_config:
        import torch

        import ionization_gb300 as ig

        torch.cuda.set_device(local_rank)
        ig.build()
        print(json.dumps(run_per_config(args, measured_peaks()[0])), flush=True)
        return
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        out = run_ours(args, rank, world, local_rank)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
