"""Edge shapes: meshes smaller than a chunk, a tile or a warp (one l, lines
of a few points, 2D meshes a few points wide), complex128 against the
oracle on the same inputs."""

import copy

import numpy as np
import pytest

from oracle import mesh as om

from .conftest import load_golden, rel_l2
from .specs import product_spec

pytestmark = pytest.mark.gpu


def _run_both(kind, params):
    want = om.run_from_params(kind, params)
    sim = product_spec(kind, params).to_sim()
    sim.run()
    return sim, want


def _check(sim, want, tol=1e-10):
    assert rel_l2(np.asarray(sim.mesh.g), want["g_final"]) < tol
    np.testing.assert_allclose(sim.data.norm, want["norm"], rtol=0, atol=tol)


@pytest.mark.parametrize("nr,L", [(9, 1), (17, 2), (33, 3), (40, 2)])
def test_tiny_spherical_harmonic(cuda, nr, L):
    params, _ = load_golden("sh_split_small_evenL")
    p = copy.deepcopy(params)
    p.update(r_points=nr, l_bound=L, r_bound=0.125 * (nr - 1), time_final=2.0, store_data_every=20)
    r_max = p["r_bound"] + 0.0625
    p["mask"] = dict(inner_radius=0.7 * r_max, outer_radius=r_max, smoothness=8)
    p["test_states"] = [[1, 0]] + ([[2, 1]] if L > 1 else [])
    sim, want = _run_both("sh", p)
    _check(sim, want)


@pytest.mark.parametrize("n,method", [(3, "SplitInteractionOperator"), (5, "AlternatingDirectionImplicit"),
                                      (17, "SplitInteractionOperator"), (33, "AlternatingDirectionImplicit")])
def test_tiny_line(cuda, n, method):
    params, _ = load_golden("line_split_small")
    p = copy.deepcopy(params)
    p.update(z_points=n, z_bound=2.0 * n, method=method, time_final=1.0, store_data_every=5)
    p["mask"] = dict(inner_radius=1.5 * n, outer_radius=2.0 * n, smoothness=8)
    sim, want = _run_both("line", p)
    _check(sim, want)


@pytest.mark.parametrize("nz,nx", [(4, 3), (9, 16), (33, 8)])
def test_tiny_rectangle(cuda, nz, nx):
    params, _ = load_golden("rect_adi_small")
    p = copy.deepcopy(params)
    p.update(z_points=nz, x_points=nx, time_final=0.5)
    sim, want = _run_both("rect", p)
    _check(sim, want)
