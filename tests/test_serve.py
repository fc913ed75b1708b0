"""Served form (continuous batching): results must not depend on the mix.

A request served together with others — different mesh kinds, sizes,
precisions and step counts, admitted and retired at different chunks — gives
bit-identical psi and data to the same request served alone, and a served
complex128 request equals the plain mesh path (spec.to_sim().run())."""

import numpy as np
import pytest

from ionization_gb300 import workloads


def test_poisson_mix_is_seeded_and_in_range():
    a = workloads.poisson_scan_parameters(200, seed=5)
    b = workloads.poisson_scan_parameters(200, seed=5)
    assert a == b
    arr = np.array([p["arrival"] for p in a])
    assert np.all(np.diff(arr) > 0)
    assert 5.0 < arr[-1] < 15.0  # 200 arrivals at 20 per second
    lines = [p for p in a if p["kind"] == "line"]
    shs = [p for p in a if p["kind"] == "sh"]
    assert lines and shs
    assert all(2048 <= p["points"] <= 16384 for p in lines)
    assert all(1000 <= p["points"] <= 4000 and 21 <= p["l_bound"] <= 101 for p in shs)
    assert all(2000 <= p["steps"] <= 50000 for p in a)
    frac64 = np.mean([p["precision"] == "c64x" for p in a])
    assert 0.7 < frac64 < 0.9


def _small_requests():
    from ionization_gb300.serve import Request

    return [
        Request(0, 0.0, "sh", "c64", 150, 400, 21, 0.05, 0.1, 3, 0.2),
        Request(1, 0.0, "line", "c128", 90, 2048, 0, 0.03, 0.08, 2, 1.0),
        Request(2, 0.0, "sh", "c128", 60, 300, 30, 0.02, 0.15, 4, 2.0),
        Request(3, 0.0, "line", "c64", 130, 9000, 0, 0.05, 0.057, 3, 0.0),  # a two-CTA cluster
        Request(4, 0.0, "sh", "c64", 40, 1000, 25, 0.08, 0.06, 2, 3.0),
        Request(5, 0.0, "line", "c128", 70, 5000, 0, 0.04, 0.12, 2, 0.5),  # a two-CTA cluster
        Request(6, 0.0, "sh", "c64x", 50, 500, 15, 0.06, 0.09, 2, 1.5),
        Request(7, 0.0, "line", "c64x", 60, 6000, 0, 0.05, 0.1, 2, 0.7),  # residual form, two-CTA cluster
    ]


@pytest.mark.gpu
def test_served_mix_equals_each_request_alone(cuda):
    from ionization_gb300.serve import Server

    reqs = _small_requests()
    mixed = {c.request.id: c for c in Server(chunk_steps=16, keep_psi=True).run(reqs, realtime=False)}
    assert sorted(mixed) == [r.id for r in reqs]
    for r in reqs:
        # same chunk length: every simulation meets its chunk boundaries at the
        # same steps of its own run, whatever else is in the batch; complex128
        # results do not depend on the chunk length at all
        chunks = (16, 7) if r.precision == "c128" else (16,)
        for chunk in chunks:
            (alone,) = Server(chunk_steps=chunk, keep_psi=True).run([r], realtime=False)
            m = mixed[r.id]
            np.testing.assert_array_equal(m.psi, alone.psi)
            np.testing.assert_array_equal(m.norm, alone.norm)
            np.testing.assert_array_equal(m.inner_products, alone.inner_products)


@pytest.mark.gpu
def test_served_c128_equals_plain_mesh_path(cuda):
    from ionization_gb300.serve import Server

    reqs = [r for r in _small_requests() if r.precision == "c128"]
    served = {c.request.id: c for c in Server(chunk_steps=16, keep_psi=True).run(reqs, realtime=False)}
    for r in reqs:
        sim = r.spec().to_sim()
        sim.run()
        np.testing.assert_array_equal(served[r.id].psi, np.asarray(sim.mesh.g))
        np.testing.assert_array_equal(served[r.id].norm, sim.data.norm)


@pytest.mark.gpu
def test_hbm_budget_limits_admission(cuda):
    from ionization_gb300.serve import Server, device_bytes

    reqs = _small_requests()
    need = sorted(device_bytes(r) for r in reqs)
    budget = need[0] + need[1] - 1  # no two requests fit together
    server = Server(hbm_budget=budget, chunk_steps=16)
    done = server.run(reqs, realtime=False)
    assert len(done) == len(reqs)  # one that exceeds the budget alone still runs, alone
    assert server.peak_active == 1

    roomy = Server(hbm_budget=sum(need), chunk_steps=16)
    assert len(roomy.run(reqs, realtime=False)) == len(reqs)
    assert roomy.peak_active == len(reqs)
    assert roomy.peak_bytes == sum(need)
    assert roomy.peak_allocated_bytes <= roomy.peak_bytes


@pytest.mark.gpu
def test_device_bytes_bounds_the_allocation(cuda):
    from ionization_gb300 import _device as dev
    from ionization_gb300.core import Precision
    from ionization_gb300.serve import device_bytes, host_tables

    for r in _small_requests():
        tab = host_tables(r)
        d = (dev.ShDeviceSim if r.kind == "sh" else dev.LineDeviceSim)(tab, Precision(r.precision))
        assert d.nbytes() <= device_bytes(r), r
