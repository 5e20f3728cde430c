"""The marching-cubes restatement of the oracle (CPU): on a sphere SDF the
mesh is a closed, consistently oriented 2-manifold whose triangles face
outward, with the sphere's area; every case of the table closes its loops."""
import numpy as np

from oracle import mcubes as M


def _edges_of(faces):
    out = {}
    for a, b, c in faces:
        for u, v in ((a, b), (b, c), (c, a)):
            out[(int(u), int(v))] = out.get((int(u), int(v)), 0) + 1
    return out


def test_table_cases():
    assert M.TABLE[0] == [] and M.TABLE[255] == []
    assert max(len(t) for t in M.TABLE) == 5
    for case, tris in enumerate(M.TABLE):
        # each crossing edge of the cube appears in the case's loops
        crossing = {e for e, (a, b) in enumerate(M.EDGES) if ((case >> a) & 1) != ((case >> b) & 1)}
        assert {e for t in tris for e in t} == crossing, case


def test_sphere_is_closed_outward_and_has_the_area():
    n, r = 28, 9.3
    ax = np.arange(n, dtype=np.float32)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    c = np.array([13.2, 13.9, 12.6], np.float32)
    sdf = (np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - r).astype(np.float32)
    v, f = M.marching_cubes(sdf, 0.0)
    e = _edges_of(f)
    assert all(k == 1 for k in e.values())                       # manifold, consistent
    assert all((b, a) in e for (a, b) in e)                      # closed
    nrm = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
    assert np.all((nrm * (v[f].mean(1) - c)).sum(1) > 0)        # outward
    area = 0.5 * np.linalg.norm(nrm, axis=1).sum()
    assert abs(area / (4 * np.pi * r * r) - 1) < 0.01
    assert np.abs(np.linalg.norm(v - c, axis=1) - r).max() < 0.05


def test_array_form_equals_the_loop_form():
    """marching_cubes_vec (the CPU baseline's form) gives the loop form's mesh
    bit for bit: random lattices whose sizes are not multiples of anything,
    and a sphere."""
    rng = np.random.default_rng(4)
    for shape, lv in [((2, 2, 2), 0.0), ((9, 13, 7), 0.1), ((5, 6, 33), -0.2)]:
        g = rng.normal(size=shape).astype(np.float32)
        a = M.marching_cubes(g, lv, (-0.7, 0.2, 1.5), (0.01, 0.02, 0.03))
        b = M.marching_cubes_vec(g, lv, (-0.7, 0.2, 1.5), (0.01, 0.02, 0.03))
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    n = 24
    ax = np.arange(n, dtype=np.float32)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    sdf = (np.sqrt((X - 11.3) ** 2 + (Y - 12.1) ** 2 + (Z - 11.7) ** 2) - 8.4).astype(np.float32)
    a, b = M.marching_cubes(sdf, 0.0), M.marching_cubes_vec(sdf, 0.0)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
