"""Marching cubes on the GPU (angelo_mc_*) against the CPU restatement
(oracle/mcubes.py): identical vertices (bit-exact float32) and faces on
random lattices and a sphere; the geometry's isosurface() on the sphere-
initialised VolumeSDF lies on the 0.5 sphere."""
import numpy as np
import pytest
import torch

from oracle import mcubes as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


@pytest.mark.parametrize("shape,level", [((2, 2, 2), 0.0), ((9, 13, 7), 0.1), ((23, 17, 20), -0.3),
                                         ((3, 4, 33), 0.1), ((4, 3, 64), -0.2), ((5, 6, 70), 0.0),
                                         ((2, 5, 31), 0.3)])
def test_random_lattice_matches_oracle(dev, shape, level):
    from angelo_gb import mesh
    g = np.random.default_rng(sum(shape)).normal(size=shape).astype(np.float32)
    origin, spacing = (-0.7, 0.2, 1.5), (0.01, 0.02, 0.03)
    v, f = mesh.marching_cubes(torch.from_numpy(g).to(dev), level, origin, spacing)
    rv, rf = M.marching_cubes(g, level, origin, spacing)
    np.testing.assert_array_equal(v.cpu().numpy(), rv)
    np.testing.assert_array_equal(f.cpu().numpy(), rf)


def test_sphere_matches_oracle_and_is_closed(dev):
    from angelo_gb import mesh
    n, r = 48, 17.1
    ax = np.arange(n, dtype=np.float32)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    c = np.array([23.2, 24.7, 22.9], np.float32)
    sdf = (np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r).astype(np.float32)
    v, f = mesh.marching_cubes(torch.from_numpy(sdf).to(dev), 0.0)
    rv, rf = M.marching_cubes(sdf, 0.0)
    np.testing.assert_array_equal(v.cpu().numpy(), rv)
    np.testing.assert_array_equal(f.cpu().numpy(), rf)
    fv = f.cpu().numpy()
    edges = set()
    for a, b, cc in fv:
        for e in ((a, b), (b, cc), (cc, a)):
            assert e not in edges
            edges.add(e)
    assert all((b, a) in edges for (a, b) in edges)


def test_isosurface_of_the_sphere_initialised_field(dev):
    """isosurface() (models/geometry.py:144-149): the sphere-initialised
    field's lattice at resolution 128 triangulated at the 0.001 level; the
    vertices lie on that level set of the field itself (linear
    interpolation inside a cell of 2/128) and the mesh is closed."""
    from angelo_gb import models, workloads
    cfg = workloads.model_config("small")
    cfg["geometry"]["isosurface"] = dict(method="mc", resolution=128)
    m = models.make("neus", cfg).to(dev)
    m.update_step(0, 0)
    mesh = m.isosurface()
    v, f = mesh["v_pos"], mesh["t_pos_idx"].numpy()
    assert len(f) > 1000
    with torch.no_grad():
        level = m.geometry.forward_level(v.to(dev)).cpu().numpy()
    assert np.abs(level - 0.001).max() < 5e-3, np.abs(level - 0.001).max()
    edges = {(int(a), int(b)) for t in f for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0]))}
    assert len(edges) == 3 * len(f) and all((b, a) in edges for a, b in edges)
