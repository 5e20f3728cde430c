"""The oracle, pinned: against the golden vectors produced by the reference's own
model code, and against known answers for the restated tcnn / nerfacc
arithmetic (for which the reference ships no tests or fixtures)."""
import math

import numpy as np
import pytest
import torch

from oracle import cref
from oracle import neus_fp64 as O
from golden_util import NAMES, load, oracle_cfgs, params


def _oracle_forward_backward(g):
    G, T = oracle_cfgs(g)
    P = params(g)
    for v in P.values():
        v.requires_grad_(True)
    rays = torch.tensor(g["rays"], dtype=torch.float64)
    c = g["cfg"]
    binary = (np.unpackbits(g["occ_bits"], bitorder="little").reshape(128, 128, 128)
              if c["grid_prune"] else np.ones((1, 1, 1), np.uint8))
    roi = (g["param/scene_aabb"] if c["grid_prune"]
           else np.array([-1e10] * 3 + [1e10] * 3, np.float32))
    step = 1.732 * 2 * c["radius"] / c["num_samples_per_ray"]
    _, offsets, ri, t0, t1, _ = cref.march(g["rays"][:, :3], g["rays"][:, 3:], g["t_min"],
                                           g["t_max"], roi, binary, step)
    out = O.neus_render(rays, P, G, T, (offsets, ri, t0, t1),
                        torch.tensor(g["rand_dirs"], dtype=torch.float64),
                        float(g["cos_anneal_ratio"]), torch.tensor(g["background"]))
    l_main, l_curv = O.neus_loss_terms(out, torch.tensor(g["target"], dtype=torch.float64))
    l_main.backward(retain_graph=True)
    grads = {k: p.grad.detach().numpy().copy() for k, p in P.items() if p.grad is not None}
    for p in P.values():
        p.grad = None
    l_curv.backward()
    grads_curv = {k: p.grad.detach().numpy().copy() for k, p in P.items() if p.grad is not None}
    return out, (l_main + l_curv).item(), grads, grads_curv, offsets


def _check_grads(got, g, prefix, tol):
    """Max error per parameter relative to that parameter's largest gradient,
    floored at 1e-4 of the largest gradient of any parameter (a gradient that
    is zero in exact arithmetic shows float32 noise in the golden)."""
    n = 0
    gmax = max(np.abs(g[k]).max() for k in g if k.startswith(prefix))
    for k, v in got.items():
        if prefix + k not in g:
            continue
        ref = g[prefix + k]
        scale = max(np.abs(ref).max(), 1e-4 * gmax)
        err = np.abs(v.reshape(ref.shape) - ref).max() / scale
        assert err < tol, (prefix + k, err)
        n += 1
    assert n > 0


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_golden(name):
    g = load(name)
    out, loss, grads, grads_curv, offsets = _oracle_forward_backward(g)
    # integer outputs of the march are exact
    np.testing.assert_array_equal(offsets, g["offsets"])
    np.testing.assert_array_equal(out["ray_indices"].numpy(), g["out/ray_indices"])
    # float outputs: the reference ran in float32, the oracle in float64
    tol = dict(rtol=2e-4, atol=2e-5)
    for k in ("comp_rgb", "opacity", "depth", "comp_rgb_full", "sdf_samples", "weights",
              "points", "intervals"):
        np.testing.assert_allclose(out[k].detach().numpy().reshape(g["out/" + k].shape),
                                   g["out/" + k], **tol, err_msg=k)
    # finite differences of float32 values: looser, scaled by the stencil
    np.testing.assert_allclose(out["sdf_grad_samples"].detach().numpy(), g["out/sdf_grad_samples"],
                               rtol=2e-3, atol=2e-3)
    np.testing.assert_allclose(out["comp_normal"].detach().numpy(), g["out/comp_normal"],
                               rtol=1e-3, atol=1e-3)
    lap_o = out["sdf_laplace_samples"].detach().numpy()
    assert np.mean(np.abs(lap_o - g["out/sdf_laplace_samples"])) < 2e-3
    assert abs(loss - float(g["loss"])) < 1e-4 * max(1.0, abs(float(g["loss"])))
    # parameter gradients of rgb MSE + eikonal (well conditioned)
    assert np.abs(g["grad/geometry.encoding.encoding.encoding.params"]).max() > 0
    _check_grads(grads, g, "grad/", 2e-3)
    # the curvature gradient only where the shifted stencil stays in the box
    if g["cfg"]["radius"] >= 1.0:
        _check_grads(grads_curv, g, "grad_curv/", 2e-2)


def test_hash_index_known_answers():
    # config-1 table: 8 levels, 2^16 entries, base 16, scale 1.5
    off, res, sc = cref.hashgrid_layout(8, 16, 16, 1.5)
    # scale_l = exp2f(l * log2f(1.5)) * 16 - 1 in float32: within a few ulp of
    # 16 * 1.5^l - 1 (log2f(1.5) is rounded, so levels >= 5 are not exact)
    np.testing.assert_allclose(sc, np.array([16 * 1.5 ** l - 1 for l in range(8)]), rtol=4e-7)
    assert list(sc[:5]) == [15.0, 23.0, 35.0, 53.0, 80.0]
    np.testing.assert_array_equal(res, np.ceil(sc).astype(np.uint32) + 1)
    # levels 0..2 are dense (res^3 <= 2^16, aligned to 8), the rest hashed
    assert list(np.diff(off)[:3]) == [16 ** 3, 24 ** 3, 36 ** 3]
    assert all(v == 1 << 16 for v in np.diff(off)[3:])
    # a point whose level-0 cell is (3, 5, 7): pos = 15 * x + 0.5
    x = np.array([[3.0 / 15, 5.0 / 15, 7.0 / 15]], np.float32)
    idx, w, cells = cref.hashgrid_index(x, (off, res, sc), with_cells=True)
    g0 = cells[0, 0]
    assert list(g0) == [3, 5, 7]
    assert idx[0, 0, 0] == 3 + 5 * 16 + 7 * 256          # dense corner (0,0,0)
    assert idx[0, 0, 7] == 4 + 6 * 16 + 8 * 256          # corner (+1,+1,+1)
    # hashed level 3: XOR of coordinate * prime, modulo 2^16
    c3 = cells[0, 3].astype(np.uint64)
    h = (int(c3[0]) * 1) ^ ((int(c3[1]) * 2654435761) & 0xFFFFFFFF) ^ \
        ((int(c3[2]) * 805459861) & 0xFFFFFFFF)
    assert idx[0, 3, 0] == h % (1 << 16)
    # trilinear weights sum to one
    xs = np.random.default_rng(0).random((1000, 3), dtype=np.float32)
    _, w = cref.hashgrid_index(xs, (off, res, sc))
    np.testing.assert_allclose(w.sum(-1), 1.0, atol=1e-6)


def test_finest_level_of_the_full_table_is_hashed():
    # 16 levels, 2^22, base 32, finest 2048: float32 scale of level 15 is just
    # above 2047, so the resolution is 2049 and the level hashes (a float64
    # scale of exactly 2047 would give 2048^2 = 2^22 and a wrapped stride).
    off, res, sc = cref.hashgrid_layout(16, 22, 32, 1.3195079107728942)
    assert res[15] == 2049 and sc[15] > 2047.0
    assert list(res[:6]) == [32, 43, 56, 74, 98, 129]
    dense = [l for l in range(16) if int(res[l]) ** 3 <= 1 << 22]
    assert dense == [0, 1, 2, 3, 4, 5]


def test_encode_is_trilinear_in_the_table():
    lay = O.HashGridLayout(8, 2, 12, 16, 1.5)
    rng = np.random.default_rng(1)
    t = rng.uniform(-1, 1, lay.n_params).astype(np.float32)
    x = rng.random((300, 3), dtype=np.float32)
    e1 = cref.hashgrid_encode(x, t, lay.cref_layout)
    e2 = cref.hashgrid_encode(x, 2 * t, lay.cref_layout)
    np.testing.assert_array_equal(e2, 2 * e1)          # scaling by 2 is exact
    e64 = O.hash_encode(torch.tensor(x, dtype=torch.float64), torch.tensor(t, dtype=torch.float64),
                        lay).numpy()
    # float32 positions at the finest level (scale 272) carry ~3e-5 of weight error
    np.testing.assert_allclose(e1, e64, rtol=1e-5, atol=1e-4)
    # band mask: levels >= active produce zeros
    e_m = cref.hashgrid_encode(x, t, lay.cref_layout, active_levels=3)
    assert np.all(e_m[:, 6:] == 0) and np.array_equal(e_m[:, :6], e1[:, :6])


def test_sh4_orthonormal():
    # Monte-Carlo check of orthonormality of the 16 real SH on the sphere
    rng = np.random.default_rng(2)
    v = rng.normal(size=(200000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    Y = cref.sh4(((v + 1) / 2).astype(np.float32))
    gram = Y.T @ Y * (4 * math.pi / len(v))
    np.testing.assert_allclose(gram, np.eye(16), atol=3e-2)


def test_fd_gradient_of_analytic_sphere():
    # FD stencil of models/geometry.py:219-234 on sdf = |x| - 0.5: |grad| = 1 + O(eps^2)
    eps = 1e-2
    p = torch.tensor(np.random.default_rng(3).uniform(-0.8, 0.8, (500, 3)))
    p = p[(p.norm(dim=1) > 0.2)]
    off = torch.tensor(O._FD_OFFSETS, dtype=torch.float64) * eps
    pd = p[:, None, :] + off
    sd = pd.norm(dim=-1) - 0.5
    grad = 0.5 * (sd[:, 0::2] - sd[:, 1::2]) / eps
    assert torch.allclose(grad.norm(dim=-1), torch.ones(len(p), dtype=torch.float64), atol=1e-3)


def test_alpha_closed_form():
    # sdf = 0 at a head-on sample (cos = -1, ratio 1): alpha = (s(a) - s(-a) + 1e-5)/(s(a)+1e-5)
    s, dist = torch.tensor(20.0, dtype=torch.float64), 0.05
    a = O.get_alpha(torch.zeros(1, dtype=torch.float64), torch.tensor([[0.0, 0, 1]]).double(),
                    torch.tensor([[0.0, 0, -1]]).double(), torch.tensor([dist], dtype=torch.float64), s, 1.0)
    sig = lambda v: 1 / (1 + math.exp(-v))  # noqa: E731
    pc, nc = sig(dist / 2 * 20), sig(-dist / 2 * 20)
    assert abs(a.item() - (pc - nc + 1e-5) / (pc + 1e-5)) < 1e-12


def test_transmittance_of_constant_alpha():
    a = np.full(40, 0.1, np.float32)
    w, t = cref.weights(a, np.array([0, 40]), early_stop_eps=0.0)
    np.testing.assert_allclose(t, 0.9 ** np.arange(40), rtol=1e-5)
    np.testing.assert_allclose(w, 0.1 * 0.9 ** np.arange(40), rtol=1e-5)
    # early stop: once T < 1e-4 every later weight is zero
    a = np.full(200, 0.5, np.float32)
    w, t = cref.weights(a, np.array([0, 200]))
    k = int(np.argmax(t < 1e-4))
    assert k > 0 and np.all(w[k:] == 0) and np.all(w[:k] > 0)


def test_empty_occupancy_grid_gives_no_samples():
    rays = np.array([[0, 0, -3, 0, 0, 1], [0.1, 0.2, 3, 0, 0, -1]], np.float32)
    tmin, tmax = cref.ray_aabb(rays[:, :3], rays[:, 3:], np.array([-1, -1, -1, 1, 1, 1], np.float32))
    np.testing.assert_allclose(tmin, [2, 2]) and np.testing.assert_allclose(tmax, [4, 4])
    counts, off, ri, t0, t1, ovf = cref.march(rays[:, :3], rays[:, 3:], tmin, tmax,
                                              np.array([-1, -1, -1, 1, 1, 1], np.float32),
                                              np.zeros((8, 8, 8), np.uint8), 0.01)
    assert counts.sum() == 0 and len(ri) == 0 and not ovf
    counts, off, ri, t0, t1, ovf = cref.march(rays[:, :3], rays[:, 3:], tmin, tmax,
                                              np.array([-1, -1, -1, 1, 1, 1], np.float32),
                                              np.ones((8, 8, 8), np.uint8), 0.01)
    assert list(counts) == [200, 200]
    assert np.all(np.diff(t0[:200]) > 0) and np.all(ri[:200] == 0) and np.all(ri[200:] == 1)


def test_missing_ray_gets_far_sentinel():
    tmin, tmax = cref.ray_aabb(np.array([[5, 5, 5]], np.float32), np.array([[1, 0, 0]], np.float32),
                               np.array([-1, -1, -1, 1, 1, 1], np.float32))
    assert tmin[0] == np.float32(1e10) and tmax[0] == np.float32(1e10)


def test_ide_matches_reference_golden():
    """The oracle's integrated directional encoding (associated-Legendre
    recurrence) against the reference's generate_ide_fn(4) (golden vectors
    from tests/golden/make_ide_golden.py, float32 as the reference computes)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ide_deg4.npz"))
    out = O.ide(torch.from_numpy(g["xyz"]).double(), torch.from_numpy(g["kappa_inv"]).double(), 4)
    assert out.shape == (96, 38)
    np.testing.assert_allclose(out.numpy(), g["ide"], rtol=1e-5, atol=1e-5)
