"""Batched form (ionization_gb300.batch): simulations of different sizes,
pulses, step counts and data cadences advanced together give, each, exactly
what the same simulation gives on the plain mesh path (spec.to_sim().run()):
the kernels' arithmetic on a line or a row tile does not depend on its
batch-mates.  The bulk readback (psi_all, results) equals the per-simulation
one."""

import numpy as np
import pytest

from ionization_gb300 import workloads as wl


def _specs(precision):
    # (r_points, l_bound, E0, omega, cycles, cep, steps, store_data_every)
    shapes = [
        (300, 12, 0.05, 0.1, 2, 0.0, 40, -1),
        (170, 7, 0.08, 0.06, 2, 1.0, 55, 5),
        (520, 21, 0.03, 0.2, 3, 0.3, 33, 4),
        (96, 3, 0.1, 0.15, 1, 2.0, 17, -1),
    ]
    return [wl.sh_spec(f"batch_{k}", *p[:7], precision=precision, store_data_every=p[7],
                       mask_width=0.4 * wl.DR * p[0])
            for k, p in enumerate(shapes)]


def test_batch_specs_are_uneven():
    specs = _specs("c128")
    assert len({s.r_points for s in specs}) == len(specs)
    assert len({s.time_final for s in specs}) == len(specs)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["c128", "c64x", "c64"])
def test_batch_equals_each_simulation_alone(cuda, precision):
    from ionization_gb300 import batch as bm

    b = bm.BatchedSphericalHarmonicSimulation(_specs(precision), graph_steps=8)
    b.run()
    res = b.results()
    psis = b.psi_all()
    for k, spec in enumerate(_specs(precision)):
        sim = spec.to_sim()
        sim.run()
        want = np.asarray(sim.mesh.g)
        np.testing.assert_array_equal(psis[k], want)
        np.testing.assert_array_equal(b.psi(k), want)
        np.testing.assert_array_equal(res[k]["norm"], sim.data.norm)
        got = list(res[k]["inner_products"].values())  # in test-state order
        for v, st in zip(got, sim.spec.test_states, strict=True):
            np.testing.assert_array_equal(v, sim.data.inner_products[st])


@pytest.mark.gpu
def test_autotune_times_every_candidate(cuda):
    from ionization_gb300 import _device as dev
    from ionization_gb300 import batch as bm

    best, timings = bm.autotune(_specs("c64x"), precision="c64x", graph_steps=(4, 8), steps=8)
    rows = dev.SH_ROWS_CHOICES[dev.Precision.C64X]
    assert {f"rows{r}_graph8" for r in rows} <= set(timings)
    assert best["rows"] in rows and best["graph_steps"] in (4, 8)
    # the per-bucket stage: every other row count for every bucket
    n_buckets = len(bm._bucket_lines("c64x", [bm._host_tables(s)[0] for s in _specs("c64x")], best["rows"]))
    assert len(best["bucket_rows"]) == n_buckets
    assert all(r == 0 or r in rows for r in best["bucket_rows"])
    per_bucket = [k for k in timings if "_b" in k]
    assert len(per_bucket) >= n_buckets
    extra = "".join(f"_b{b}r{r}" for b, r in enumerate(best["bucket_rows"]) if r)
    assert f"rows{best['rows']}_graph{best['graph_steps']}{extra}" in timings
    assert all(v > 0 for v in timings.values())


@pytest.mark.gpu
def test_bucket_rows_per_bucket(cuda):
    """Buckets launched at their own rows per thread (16 for the longest
    lines, 4 for the next): each bucket's CTA is sized for its lines at its
    rows, and the populations equal the single-shape plan's to 1e-8
    (measured 1.3e-9: the partition changes where the solve rounds, not what
    it solves)."""
    from ionization_gb300 import batch as bm

    base = bm.BatchedSphericalHarmonicSimulation(_specs("c64x"), graph_steps=8)
    mixed = bm.BatchedSphericalHarmonicSimulation(_specs("c64x"), graph_steps=8, bucket_rows=(16, 4))
    shape = bm.plan_shape(mixed)["radial_buckets"]
    assert [b["rows_per_thread"] for b in shape] == [16, 4, 8]
    nr = sorted((s.r_points for s in _specs("c64x")), reverse=True)
    assert shape[0]["threads"] == 64 and shape[0]["threads"] * 16 >= nr[0]
    assert shape[1]["threads"] >= -(-nr[1] // 4)
    base.run()
    mixed.run()
    for a, b in zip(base.results(), mixed.results(), strict=True):
        assert abs(a["initial_state_overlap"][-1] - b["initial_state_overlap"][-1]) < 1e-8
        np.testing.assert_allclose(a["norm"], b["norm"], rtol=0, atol=1e-8)


@pytest.mark.gpu
def test_full_sweep_c64x_populations_match_c128(cuda):
    """The full 512-simulation uneven sweep (Nr 800-3200, l_max 20-80, 52.3 M
    points), 64 steps: every simulation's final ground-state population in
    the c64x form is within 1e-7 of the complex128 batch, and no norm grows
    beyond rounding (the step is unitary and the mask only absorbs): 1e-12
    in complex128 (measured 4e-15), 1e-8 in c64x (measured 5e-9: the FP32
    rotation coefficients satisfy cos^2 + sin^2 = 1 only to ~1e-7 a^2, a
    pseudo-random error per pair and step)."""
    from ionization_gb300 import batch as bm

    out = {}
    for prec in ("c128", "c64x"):
        specs = wl.uneven_sh_sweep(512, steps=64, precision=prec)
        b = bm.BatchedSphericalHarmonicSimulation(specs, graph_steps=32)
        b.run()
        out[prec] = b.results()
        del b
    p128 = np.array([r["initial_state_overlap"][-1] for r in out["c128"]])
    p64 = np.array([r["initial_state_overlap"][-1] for r in out["c64x"]])
    assert np.all(np.isfinite(p64)) and len(p64) == 512
    assert np.max(np.abs(p64 - p128)) < 1e-7
    for prec, tol in (("c128", 1e-12), ("c64x", 1e-8)):
        norms = np.array([r["norm"] for r in out[prec]])
        growth = float(np.max(norms[:, -1] / norms[:, 0] - 1))
        print(f"{prec}: largest norm growth over 64 steps {growth:.2e}")
        assert growth < tol


# the sweep's most strongly driven simulations (E0 0.07-0.1, omega 0.13-0.19,
# 6-10 cycles, ionization up to 40 %): where the FP32 rounding of the radial
# Hamiltonian moved the final populations by up to 5e-6 before the refinement
# formed its residual with the FP64 row sums
STRONG = [146, 145, 426, 418, 508, 224, 95, 471]


@pytest.mark.gpu
@pytest.mark.parametrize("rows", [4, 8])
def test_strongly_driven_c64x_populations_match_c128(cuda, rows):
    """Over the whole 10000-step run, the c64x form's final ground-state
    population and ionization probability stay within 3e-7 of the complex128
    batch on the sweep's most strongly driven simulations, at 4 and 8 rows
    per thread of the radial solve."""
    from ionization_gb300 import batch as bm

    out = {}
    for prec, r in (("c128", 0), ("c64x", rows)):
        specs = wl.uneven_sh_sweep(512, steps=10000, precision=prec, subset=STRONG)
        b = bm.BatchedSphericalHarmonicSimulation(specs, graph_steps=64, cn_rows=r)
        b.run()
        out[prec] = b.results()
        del b
    pg = {k: np.array([r["initial_state_overlap"][-1] for r in v]) for k, v in out.items()}
    pb = {k: np.array([r["bound_state_overlap"][-1] for r in v]) for k, v in out.items()}
    assert np.max(1 - pb["c128"]) > 0.3  # strongly driven indeed
    dg = np.abs(pg["c64x"] - pg["c128"])
    di = np.abs(pb["c64x"] - pb["c128"])
    print(f"rows {rows}: max |dP_ground| {dg.max():.2e}, max |dP_ion| {di.max():.2e}")
    assert dg.max() < 3e-7 and di.max() < 3e-7


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["c64x", "c128"])
def test_batches_on_two_streams_in_graphs(cuda, precision):
    """Two batches stepped through CUDA graphs on two streams at once (each
    graph forks its radial buckets onto side streams of its own capture
    stream) give, bit for bit, what each gives run alone."""
    import torch

    from ionization_gb300 import batch as bm

    specs = _specs(precision)
    sets = (specs[:2] + specs[3:], specs)  # 2 and 3 radial buckets
    alone = []
    for ss in sets:
        b = bm.BatchedSphericalHarmonicSimulation(ss, graph_steps=8)
        b.run()
        alone.append((b.psi_all(), b.results()))
    batches = [bm.BatchedSphericalHarmonicSimulation(ss, graph_steps=8) for ss in sets]
    assert [len(bm.plan_shape(b)["radial_buckets"]) for b in batches] == [2, 3]
    streams = [torch.cuda.Stream() for _ in batches]
    for s in streams:
        s.wait_stream(torch.cuda.current_stream())
    while any(b.steps_remaining for b in batches):
        for b, s in zip(batches, streams):
            if b.steps_remaining:
                with torch.cuda.stream(s):
                    b.step(16)
    for s in streams:
        torch.cuda.current_stream().wait_stream(s)
    for b, (psis, res) in zip(batches, alone, strict=True):
        for got, want in zip(b.psi_all(), psis, strict=True):
            np.testing.assert_array_equal(got, want)
        for got, want in zip(b.results(), res, strict=True):
            np.testing.assert_array_equal(got["norm"], want["norm"])
            for k in want["inner_products"]:
                np.testing.assert_array_equal(got["inner_products"][k], want["inner_products"][k])
