"""Saving and loading simulations, as the reference's own tests do
(tests/mesh/test_save_and_load.py:10-47 in the ionization project): psi
round-trips bit for bit when the mesh is saved, a simulation saved without
its mesh loads with ``mesh`` None, and a simulation that has already dropped
its mesh can still be saved.  One specification per mesh family with a
device path."""

import numpy as np
import pytest

from .conftest import load_golden
from .specs import product_spec

CASES = [("line", "line_adi_small"), ("sh", "sh_split_small_oddL"), ("cyl", "cyl_adi_small"),
         ("rect", "rect_adi_small"), ("slice", "slice_adi_small")]


def _sim(kind, name):
    params, _ = load_golden(name)
    return product_spec(kind, params).to_sim()


def _random_g(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", CASES)
def test_loaded_sim_mesh_is_same_as_original(cuda, tmp_path, kind, name):
    from ionization_gb300.mesh import MeshSimulation

    sim = _sim(kind, name)
    special = _random_g(sim.mesh.g.shape, 7)
    sim.mesh.g = special
    path = sim.save(target_dir=str(tmp_path), save_mesh=True)
    loaded = MeshSimulation.load(path)
    assert np.array_equal(loaded.mesh.g, sim.mesh.g)
    if kind == "slice":
        # the device evolves D^-1 g (a diagonal similarity in theta that makes
        # the theta operator symmetric): g = D (D^-1 special) is special to
        # within a rounding of each factor
        np.testing.assert_allclose(loaded.mesh.g, special, rtol=4e-16, atol=0)
    else:
        assert np.array_equal(loaded.mesh.g, special)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", CASES)
def test_loaded_sim_mesh_is_none_if_not_saved(cuda, tmp_path, kind, name):
    from ionization_gb300.mesh import MeshSimulation

    sim = _sim(kind, name)
    path = sim.save(target_dir=str(tmp_path), save_mesh=False)
    assert MeshSimulation.load(path).mesh is None


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", CASES)
def test_can_save_sim_that_already_has_no_mesh(cuda, tmp_path, kind, name):
    from ionization_gb300.mesh import MeshSimulation

    sim = _sim(kind, name)
    sim.run(max_steps=3)
    norm = np.array(sim.data.norm, copy=True)
    sim.mesh = None
    path = sim.save(target_dir=str(tmp_path), save_mesh=False)
    loaded = MeshSimulation.load(path)
    assert loaded.mesh is None
    np.testing.assert_array_equal(loaded.data.norm, norm)
