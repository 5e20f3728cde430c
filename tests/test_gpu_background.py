"""The learned NeRF++ background (models/neus.py:141-203 with
models/geometry.py:152-177): the march through the 256^3 unbounded-sphere
grid against the nerfacc 0.3.3 restatement (bit-exact, both march paths),
weights from density against float64 autograd, and the background render
(colour, opacity, depth, its visibility test) and its parameter gradients
against the float64 oracle on the same samples, for the plain and the fused
foreground."""
import math

import numpy as np
import pytest
import torch

from oracle import cref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _rays(n, seed, r):
    g = np.random.default_rng(seed)
    o = g.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 2.5 * r * 2
    d = -o / np.linalg.norm(o, axis=1, keepdims=True) + g.uniform(-0.6, 0.6, (n, 3))
    d[: n // 8] *= -1.0          # some rays leave without crossing the box
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


@pytest.mark.parametrize("per_ray", [None, 400, 9])
def test_march_unbounded_sphere_bit_exact(dev, per_ray):
    from angelo_gb import _lib, ops
    r = 0.5
    o, d = _rays(3000, 31, r)
    aabb = np.array([-r, -r, -r, r, r, r], np.float32)
    ot, dt = torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev)
    _, t_exit = ops.ray_aabb_intersect(ot, dt, torch.from_numpy(aabb).to(dev))
    near = torch.where(t_exit > 1e9, torch.full_like(t_exit, 0.1), t_exit)
    jit = torch.from_numpy(np.random.default_rng(32).random(3000, dtype=np.float32)).to(dev)
    t_min = (near + jit * 0.01).contiguous()
    t_max = torch.full_like(t_min, 1e3)
    cone = 10 ** (math.log10(1e3) / 256) - 1.0
    g = np.random.default_rng(33)
    binary = (g.random(128 ** 3) < 0.4).astype(np.uint8)
    words = np.packbits(binary, bitorder="little").view(np.int32)
    ri, t0, t1, off, st = ops.march(ot, dt, t_min, t_max, 0.01, roi=aabb, res=(128, 128, 128),
                                    bits=torch.from_numpy(words).to(dev), cone_angle=cone,
                                    max_samples_per_ray=per_ray,
                                    contraction=_lib.CONTRACT_UNBOUNDED_SPHERE)
    _, roff, rri, rt0, rt1, ovf = cref.march(o, d, t_min.cpu().numpy(), t_max.cpu().numpy(), aabb,
                                             binary.reshape(128, 128, 128), 0.01, cone,
                                             contraction=1)
    np.testing.assert_array_equal(off.cpu().numpy(), roff)
    np.testing.assert_array_equal(ri.cpu().numpy(), rri)
    np.testing.assert_array_equal(t0.cpu().numpy(), rt0)
    np.testing.assert_array_equal(t1.cpu().numpy(), rt1)
    assert (int(st) & 3) == 0 and not ovf
    assert int(roff[-1]) > 3000 * 20
    if per_ray == 9:
        assert int(st) & 4   # over the bound: the second march


def test_density_weights_match_fp64(dev):
    from angelo_gb import ops
    from oracle import neus_fp64 as O
    g = np.random.default_rng(41)
    counts = g.integers(0, 60, 300)
    counts[:5] = 0
    off = np.zeros(301, np.int64)
    np.cumsum(counts, out=off[1:])
    n = int(off[-1])
    dt = g.uniform(0.001, 0.3, n).astype(np.float32)
    t0 = np.zeros(n, np.float32)
    for r in range(300):
        seg = slice(off[r], off[r + 1])
        t0[seg] = np.cumsum(np.concatenate([[0.2], dt[seg][:-1]])).astype(np.float32)
    t1 = (t0 + dt).astype(np.float32)
    sigma = np.exp(g.normal(size=n)).astype(np.float32)
    gw = g.normal(size=n).astype(np.float32)
    tt = lambda a: torch.from_numpy(a).to(dev)
    s = tt(sigma).requires_grad_(True)
    w = ops.render_weight_from_density(tt(t0), tt(t1), s, tt(off))
    (w * tt(gw)).sum().backward()
    s64 = torch.from_numpy(sigma.astype(np.float64)).requires_grad_(True)
    w64 = O.density_weights(torch.from_numpy(t0).double(), torch.from_numpy(t1).double(), s64,
                            list(off))
    (w64 * torch.from_numpy(gw).double()).sum().backward()
    np.testing.assert_allclose(w.detach().cpu().numpy(), w64.detach().numpy(), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(s.grad.cpu().numpy(), s64.grad.numpy(), rtol=1e-4, atol=1e-5)


def test_native_sampling_matches_reference_ops(dev):
    """The fused form's native sampling (angelo_sample_points, angelo_bg_points,
    angelo_bg_visibility, angelo_bg_compact) against the reference's chain of
    ops on the same samples: world points and midpoints, the points contracted
    by UN_BOUNDED_SPHERE, the trunc_exp density's alpha, nerfacc's visibility
    test (T >= 1e-4) and the kept samples gathered in order."""
    from angelo_gb import fused, ops
    from angelo_gb.geometry import contract_unbounded_sphere
    g = np.random.default_rng(43)
    n_rays, radius, bias = 500, 0.5, -1.0
    counts = g.integers(0, 90, n_rays)
    counts[:7] = 0
    off = np.zeros(n_rays + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    n = int(off[-1])
    dt = g.uniform(0.001, 0.4, n).astype(np.float32)
    t0 = np.zeros(n, np.float32)
    for r in range(n_rays):
        seg = slice(off[r], off[r + 1])
        t0[seg] = np.cumsum(np.concatenate([[0.6], dt[seg][:-1]])).astype(np.float32)
    t1 = (t0 + dt).astype(np.float32)
    ri = np.repeat(np.arange(n_rays, dtype=np.int32), counts)
    o, d = _rays(n_rays, 44, radius)
    out = g.normal(0.5, 1.5, (n, 8)).astype(np.float32)
    tt = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    o_t, d_t, ri_t, t0_t, t1_t, off_t, out_t = map(tt, (o, d, ri, t0, t1, off, out))

    pts = fused.bg_points(o_t, d_t, ri_t, t0_t, t1_t, radius)
    rl = ri_t.long()
    pos = o_t[rl] + d_t[rl] * ((t0_t + t1_t) * 0.5)[:, None]
    ref_pts = contract_unbounded_sphere(pos, radius)
    # the kernel's norm is the plain sum of squares; torch's reduction may
    # round it differently by an ulp or two
    torch.testing.assert_close(pts, ref_pts, rtol=0, atol=1e-6)

    # the foreground's world points and midpoints (angelo_sample_points): the
    # reference's expression bit for bit
    wpts, mid = fused.sample_points(o_t, d_t, ri_t, t0_t, t1_t)
    assert torch.equal(mid, (t0_t + t1_t) * 0.5) and torch.equal(wpts, pos)

    ri_k, t0_k, t1_k, pts_k, out_k, rows, koff = fused.bg_visible(out_t, bias, ri_t, t0_t, t1_t, off_t, pts)
    sigma = torch.exp(out_t[:, 0] + bias)
    alpha = 1.0 - torch.exp(-sigma * (t1_t - t0_t))
    keep = ops.transmittance_from_alpha(alpha, off_t) >= 1e-4
    kidx = keep.nonzero().squeeze(1)
    assert torch.equal(rows.long(), kidx)
    assert torch.equal(koff, ops.offsets_from_ray_indices(ri_t[kidx], n_rays))
    assert torch.equal(ri_k, ri_t[kidx]) and torch.equal(t0_k, t0_t[kidx]) and torch.equal(t1_k, t1_t[kidx])
    assert torch.equal(pts_k, pts[kidx]) and torch.equal(out_k, out_t[kidx])
    # every ray keeps a prefix; a good share of the samples is dropped
    assert 0.2 * n < kidx.numel() < 0.9 * n
    # the float64 transmittance agrees except within rounding of the threshold
    a64 = 1.0 - np.exp(-np.exp(out[:, 0].astype(np.float64) + bias) * (t1 - t0).astype(np.float64))
    T64 = np.ones(n)
    for r in range(n_rays):
        seg = slice(off[r], off[r + 1])
        T64[seg] = np.concatenate([[1.0], np.cumprod(1.0 - a64[seg])[:-1]])
    differ = (T64 >= 1e-4) != keep.cpu().numpy()
    assert np.all(np.abs(T64[differ] / 1e-4 - 1.0) < 1e-4)


def test_fused_density_composite_matches_fp64(dev):
    """The fused background compositing (weights from density, opacity,
    depth, colour and the background blend in one kernel each way) against
    float64 autograd of the same formulas, with empty and long rays."""
    from angelo_gb import fused
    from oracle import neus_fp64 as O
    g = np.random.default_rng(43)
    counts = g.integers(0, 300, 200)
    counts[:4] = 0
    counts[4] = 1
    off = np.zeros(201, np.int64)
    np.cumsum(counts, out=off[1:])
    n = int(off[-1])
    dt = g.uniform(0.001, 0.2, n).astype(np.float32)
    t0 = np.zeros(n, np.float32)
    for r in range(200):
        seg = slice(off[r], off[r + 1])
        t0[seg] = np.cumsum(np.concatenate([[0.5], dt[seg][:-1]])).astype(np.float32)
    t1 = (t0 + dt).astype(np.float32)
    sigma = np.exp(g.normal(size=n) - 0.5).astype(np.float32)
    rgb = g.uniform(0, 1, (n, 3)).astype(np.float32)
    bg = np.array([0.2, 0.5, 0.8], np.float32)
    gc, go, gd = g.normal(size=(200, 3)), g.normal(size=(200, 1)), g.normal(size=(200, 1))
    tt = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
    s_, c_ = tt(sigma).requires_grad_(True), tt(rgb).requires_grad_(True)
    comp, op, dep, w = fused.density_composite(s_, c_, tt(t0), tt(t1), tt(off), tt(bg))
    ((comp * tt(gc.astype(np.float32))).sum() + (op * tt(go.astype(np.float32))).sum()
     + (dep * tt(gd.astype(np.float32))).sum()).backward()
    s64 = torch.from_numpy(sigma.astype(np.float64)).requires_grad_(True)
    c64 = torch.from_numpy(rgb.astype(np.float64)).requires_grad_(True)
    w64 = O.density_weights(torch.from_numpy(t0).double(), torch.from_numpy(t1).double(), s64, list(off))
    mid = (torch.from_numpy(t0).double() + torch.from_numpy(t1).double()) * 0.5
    ridx = torch.repeat_interleave(torch.arange(200), torch.from_numpy(counts))
    op64 = torch.zeros(200, 1, dtype=torch.float64).index_add(0, ridx, w64[:, None])
    dep64 = torch.zeros(200, 1, dtype=torch.float64).index_add(0, ridx, (w64 * mid)[:, None])
    comp64 = torch.zeros(200, 3, dtype=torch.float64).index_add(0, ridx, w64[:, None] * c64)
    comp64 = comp64 + torch.from_numpy(bg).double() * (1.0 - op64)
    ((comp64 * torch.from_numpy(gc)).sum() + (op64 * torch.from_numpy(go)).sum()
     + (dep64 * torch.from_numpy(gd)).sum()).backward()
    for a, b in ((w, w64), (op, op64), (dep, dep64), (comp, comp64)):
        np.testing.assert_allclose(a.detach().cpu().numpy(), b.detach().numpy(), rtol=2e-5, atol=2e-6)
    np.testing.assert_allclose(s_.grad.cpu().numpy(), s64.grad.numpy(), rtol=2e-4, atol=2e-5)
    np.testing.assert_allclose(c_.grad.cpu().numpy(), c64.grad.numpy(), rtol=2e-5, atol=2e-6)


def _model(dev, fused):
    from angelo_gb import models, workloads
    cfg = workloads.model_config("small", fused=fused, **workloads.background(
        n_levels=8, log2_hashmap_size=16, base_resolution=16, per_level_scale=1.5, start_level=8,
        radius=1.0))
    torch.manual_seed(0)
    m = models.make("neus", cfg).to(dev)
    m.update_step(0, 5000)
    with torch.no_grad():
        gen = torch.Generator(device="cpu").manual_seed(9)
        p = m.geometry_bg.encoding_with_network.encoding.encoding.encoding.params
        p.copy_((torch.rand(p.shape, generator=gen) * 0.2 - 0.1).to(dev))
    m.train()
    m.randomized = False
    m.background_color = torch.tensor([0.2, 0.5, 0.8], device=dev)
    return m


@pytest.mark.parametrize("fused", [False, True])
def test_background_render_and_gradients_match_fp64(dev, fused):
    from oracle import neus_fp64 as O
    m = _model(dev, fused)
    o, d = _rays(512, 51, 1.0)
    rays = torch.cat([torch.from_numpy(o), torch.from_numpy(d)], -1).to(dev)
    out = m.forward_(rays)
    off, ri, t0, t1 = m._last_march_bg
    foff, _, _, _ = m._last_march_bg_full
    assert int(off[-1]) < int(foff[-1])      # the visibility test dropped samples
    gcol = torch.randn(512, 3, generator=torch.Generator(device="cpu").manual_seed(3)).to(dev)
    m.zero_grad()
    (out["comp_rgb_bg"] * gcol).sum().backward()
    P = {k: v.detach().double().clone().requires_grad_(True) for k, v in m.state_dict().items()}
    lay = O.HashGridLayout(8, 2, 16, 16, 1.5)
    B = dict(radius=1.0, lay=lay, active_levels=8, n_layers=2, density_bias=-1.0)
    ref = O.render_bg(rays.double(), P, B, 3, (off.cpu().numpy(), ri.long(), t0, t1),
                      m.background_color.double())
    for k in ("comp_rgb", "opacity", "depth"):
        np.testing.assert_allclose(out[k + "_bg"].detach().cpu().numpy(),
                                   ref[k].detach().cpu().numpy(), rtol=2e-4, atol=2e-5, err_msg=k)
    # the full colour blends the foreground over the learned background
    full = out["comp_rgb"] + out["comp_rgb_bg"] * (1 - out["opacity"])
    np.testing.assert_allclose(out["comp_rgb_full"].detach().cpu().numpy(),
                               full.detach().cpu().numpy(), rtol=1e-6, atol=1e-6)
    (ref["comp_rgb"] * gcol.double()).sum().backward()
    names = [k for k, _ in m.named_parameters() if k.startswith(("geometry_bg", "texture_bg"))]
    ours = dict(m.named_parameters())
    for k in names:
        a, b = ours[k].grad, P[k].grad
        assert a is not None and b is not None, k
        scale = float(b.abs().max()) + 1e-12
        err = float((a.double() - b).abs().max()) / scale
        rel2 = float((a.double() - b).norm() / (b.norm() + 1e-30))
        if not fused:
            assert err < 2e-3, (k, err)
        else:
            # the fused density MLP's products carry ~2^-16 of their operands
            # (bf16x3): the few hidden units whose pre-activation sits within
            # that of zero take the other side of the ReLU than float64, each
            # moving one sample's gradient by one unit's term.  Single entries
            # then move by up to ~1e-3 of the largest; the 2-norm stays close.
            assert err < 1e-2 and rel2 < 1e-3, (k, err, rel2)
    # the dropped samples are the ones behind transmittance 1e-4 (float64
    # densities on the full march; a few may sit on the threshold)
    foff, fri, ft0, ft1 = m._last_march_bg_full
    with torch.no_grad():
        fri_l = fri.long()
        pos = rays[fri_l, :3].double() + rays[fri_l, 3:].double() * ((ft0 + ft1) * 0.5).double()[:, None]
        dens, _ = O.volume_density(pos, {k: v.detach() for k, v in P.items()}, B)
        tau = dens * (ft1 - ft0).double()
        T = torch.ones_like(tau)
        fo = foff.cpu().numpy()
        for r in range(512):
            a, b = int(fo[r]), int(fo[r + 1])
            if b > a:
                T[a:b] = torch.exp(-torch.cat([tau.new_zeros(1), torch.cumsum(tau[a:b], 0)[:-1]]))
    kept = int(off[-1])
    assert abs(int((T >= 1e-4).sum()) - kept) <= max(2, kept // 1000)
