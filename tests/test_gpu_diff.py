"""Differentiation check with the reflection texture: a camera branch on
SH(d), a reflected branch on the degree-4 integrated directional encoding of
the reflected direction (roughness sigmoid(feature 5)), blended by a
predicted weight (models/texture.py:73-146, models/utils.py:209-273).

The fused training forward/backward exercises the hand-written backward
kernels behind torch.autograd.Function: the hash-table scatter-add of
dL/dfeature (fused stencil scatter), the geometry MLP backward (tensor
cores, FD and curvature stencils recomputed from the kept encodings) and the
compositing adjoint through alpha and the log-space transmittance (reverse
scan).  Gradients of the training loss (rgb MSE x10, eikonal x0.1, curvature
x5e-4) with respect to table entries, geometry and texture weights and the
variance are compared with the float64 oracle's autograd gradient, which is
itself checked against central finite differences (h = 1e-3) of the oracle,
on 256 rays x 64 samples.

The plain path's gradients are printed beside them.  Samples that march
outside the box have every stencil tap clamped to one point: their FD
gradient is exactly zero, normalize() of it back-propagates 1e12 x the
incoming gradient, and the six identical taps' contributions cancel only in
exact arithmetic; the reference's formulation (and the plain path, which
keeps it) leaves fp32 rounding of that size in the shared weights' gradients,
while the fused backward gives coincident taps weight 0 (exact).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N_RAYS = 256
H = 1e-3


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _model(dev, fused=True, log2_table=16):
    from angelo_gb import models, workloads
    cfg = workloads.model_config("small", fused=fused)
    cfg["geometry"]["xyz_encoding_config"]["log2_hashmap_size"] = log2_table
    cfg["render_step_size"] = 4.0 / 64          # 64 samples between near 0.5 and far 4.5
    cfg["texture"] = dict(
        name="volume-dual-colorV3", input_feature_dim=13 + 6, use_ide=True, ide_degree=4,
        dir_encoding_config=dict(otype="SphericalHarmonics", degree=4),
        mlp_network_config=dict(otype="VanillaMLP", activation="ReLU", output_activation="none",
                                n_neurons=64, n_hidden_layers=2),
        weitht_network_config=dict(otype="VanillaMLP", activation="ReLU",
                                   output_activation="sigmoid", n_neurons=64, n_hidden_layers=1),
        color_activation="sigmoid")
    torch.manual_seed(0)
    m = models.make("neus", cfg).to(dev)
    m.update_step(0, 5000)
    with torch.no_grad():
        g = torch.Generator(device="cpu").manual_seed(7)
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=g) * 0.1 - 0.05).to(dev))
        # the sphere initialisation leaves the hash-feature columns of the
        # first layer at zero: give them weight so that the table matters
        wv = m.geometry.network.layers[0].weight_v
        wv[:, 3:].copy_((torch.randn(wv[:, 3:].shape, generator=g) * 0.05).to(dev))
    m.train()
    m.randomized = False
    return m


def _oracle_cfg(m):
    from oracle import neus_fp64 as O
    c = m.config
    h = c.geometry.xyz_encoding_config
    lay = O.HashGridLayout(h.n_levels, h.n_features_per_level, h.log2_hashmap_size,
                           h.base_resolution, h.per_level_scale)
    G = dict(radius=float(c.radius), eps=float(m.geometry._finite_difference_eps), lay=lay,
             active_levels=int(m.geometry.hashgrid.mask_levels),
             n_layers=c.geometry.mlp_network_config.n_hidden_layers + 1,
             feature_dim=c.geometry.feature_dim)
    T = dict(kind="v3", n_layers=3, n_weight_layers=2, weight_activation="sigmoid", ide_degree=4)
    return G, T


def _loss(out, target, valid_ray):
    rgb = out["comp_rgb_full"]
    l_rgb = ((rgb[valid_ray] - target[valid_ray]) ** 2).mean() * 10.0
    l_eik = ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean() * 0.1
    l_curv = out["sdf_laplace_samples"].abs().mean() * 5e-4
    return l_rgb + l_eik + l_curv


@pytest.mark.parametrize("log2_table", [16, 22])
def test_backward_matches_central_differences(dev, log2_table):
    """log2_table 22: the differentiation configuration's 2^22-entry table
    (the finest levels hashed), the stencil recomputed in the backward."""
    from angelo_gb.scenes import look_at_c2w, pixel_directions, rays_from
    from oracle import neus_fp64 as O
    m = _model(dev, log2_table=log2_table)
    G, T = _oracle_cfg(m)
    g = np.random.default_rng(23)
    dirs = pixel_directions(128, 128, 50.0, device=dev).reshape(-1, 3)
    c2w = torch.as_tensor(look_at_c2w((1.6, 1.2, 1.5)), dtype=torch.float32, device=dev)
    pix = torch.from_numpy(g.integers(0, dirs.shape[0], N_RAYS)).to(dev)
    rays = rays_from(dirs[pix], c2w[None].expand(N_RAYS, 3, 4)).float().contiguous()
    target = torch.from_numpy(g.uniform(0, 1, (N_RAYS, 3)).astype(np.float32)).to(dev)
    bg = torch.ones(3, device=dev)
    m.background_color = bg
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, off = m.march_rays(o, d)
    assert ri.numel() > 8000
    rd = torch.randn(ri.numel(), 3, generator=torch.Generator(device="cpu").manual_seed(3)).to(dev)
    m.geometry.curvature_dirs_fn = lambda t: rd
    valid = torch.ones(N_RAYS, dtype=torch.bool, device=dev)

    # the fused path's gradients, and the plain path's (torch autograd over the
    # library's plain kernels) on the same model state
    m.zero_grad()
    out = m.forward_(rays)
    _loss(out, target, valid).backward()
    ours = {k: p.grad.detach().double().clone() for k, p in m.named_parameters() if p.grad is not None}
    mp = _model(dev, fused=False, log2_table=log2_table)
    mp.load_state_dict(m.state_dict())
    mp.background_color = bg
    mp.geometry.curvature_dirs_fn = lambda t: rd
    mp.zero_grad()
    outp = mp.forward_(rays)
    _loss(outp, target, valid).backward()
    plain = {k: p.grad.detach().double().clone() for k, p in mp.named_parameters() if p.grad is not None}

    # float64 oracle: loss of a parameter dict
    P0 = {k: v.detach().double().clone() for k, v in m.state_dict().items()}
    march = (off.cpu().numpy(), ri.long(), t0, t1)

    def loss64(P):
        with torch.no_grad():
            r = O.neus_render(rays.double(), P, G, T, march, rd.double(), 1.0, bg.double(), training=True)
        return float(_loss(r, target.double(), valid))

    # parameters to check: the table entries with the largest gradients and
    # a few random entries of every weight tensor and the variance
    checks = []
    tk = "geometry.encoding.encoding.encoding.params"
    top = torch.topk(ours[tk].abs(), 8).indices.tolist()
    checks += [(tk, i) for i in top]
    for k in ("geometry.network.layers.0.weight_v", "geometry.network.layers.2.weight_v",
              "geometry.network.layers.2.bias", "texture.ref_network.layers.0.weight",
              "texture.cam_network.layers.4.weight", "texture.weight_network.layers.0.weight",
              "texture.weight_network.layers.2.bias"):
        n = ours[k].numel()
        big = torch.topk(ours[k].abs().view(-1), min(3, n)).indices.tolist()
        checks += [(k, i) for i in big]
    checks.append(("variance.variance", 0))

    # the oracle's own autograd gradient at the same point
    Pg = {k: v.clone().requires_grad_(True) for k, v in P0.items()}
    r = O.neus_render(rays.double(), Pg, G, T, march, rd.double(), 1.0, bg.double(), training=True)
    _loss(r, target.double(), valid).backward()

    rows = []
    for k, i in checks:
        P = {kk: vv.clone() for kk, vv in P0.items()}
        flat = P[k].view(-1)
        flat[i] += H
        lp = loss64(P)
        flat[i] -= 2 * H
        lm = loss64(P)
        fd = (lp - lm) / (2 * H)
        rows.append((k, i, float(ours[k].view(-1)[i]), float(plain[k].view(-1)[i]), fd,
                     float(Pg[k].grad.view(-1)[i])))
    print("\n(param, index, fused, plain, central FD fp64, autograd fp64)")
    for row in rows:
        print(row)
    scale = max(abs(r[5]) for r in rows)
    for k, i, a, pl, fd, ag in rows:
        floor = 1e-2 * scale
        # central differences (truncation error of h = 1e-3: up to ~4e-3 here)
        # agree with the float64 autograd gradient
        assert abs(fd - ag) <= 1e-2 * max(abs(ag), floor), (k, i, fd, ag)
        # the hand-written backward (fused) agrees with the float64 gradient
        assert abs(a - ag) <= 1e-2 * max(abs(ag), floor), ("fused", k, i, a, ag)


def test_full_model_backward_matches_fp64(dev):
    """The full model (16 levels x 2^22 table entries, two hidden layers of
    64, 65 outputs, dual-colour radiance; FD eps 1/2048 at global step 6000)
    through the fused training forward/backward: its gradients of the same
    loss on the same samples against the float64 oracle's autograd gradient
    (checked against central differences in the test above), on 64 rays
    marched through the grid's inner cells."""
    from angelo_gb import models, workloads
    from angelo_gb.scenes import look_at_c2w, pixel_directions, rays_from
    from oracle import neus_fp64 as O
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("full", fused=True)).to(dev)
    m.update_step(0, 6000)
    with torch.no_grad():
        # occupied: the cells whose centres lie within 0.35 of the origin on
        # every axis, so that no stencil or curvature tap reaches the box
        # boundary (where the reference's formulation differs from the
        # fused backward: all taps of an outside point clamp to one point)
        from angelo_gb.checkpoint import pack_bits
        res = m.occupancy_grid.res
        ctr = (torch.arange(res, dtype=torch.float32) + 0.5) / res - 0.5
        inner = ctr.abs() < 0.35
        occ = inner[:, None, None] & inner[None, :, None] & inner[None, None, :]
        m.occupancy_grid.bits.copy_(pack_bits(occ.reshape(-1)).to(dev))
        m.occupancy_grid.occs.copy_(occ.reshape(-1).float().to(dev))
        g = torch.Generator(device="cpu").manual_seed(7)
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=g) * 0.1 - 0.05).to(dev))
        wv = m.geometry.network.layers[0].weight_v
        wv[:, 3:].copy_((torch.randn(wv[:, 3:].shape, generator=g) * 0.05).to(dev))
        m.variance.variance.fill_(0.5)
    m.train()
    m.randomized = False
    n_rays = 64
    rng = np.random.default_rng(31)
    dirs = pixel_directions(64, 64, 40.0, device=dev).reshape(-1, 3)
    c2w = torch.as_tensor(look_at_c2w((0.9, 0.7, 0.9)), dtype=torch.float32, device=dev)
    pix = torch.from_numpy(rng.integers(0, dirs.shape[0], n_rays)).to(dev)
    rays = rays_from(dirs[pix], c2w[None].expand(n_rays, 3, 4)).float().contiguous()
    target = torch.from_numpy(rng.uniform(0, 1, (n_rays, 3)).astype(np.float32)).to(dev)
    bg = torch.ones(3, device=dev)
    m.background_color = bg
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, off = m.march_rays(o, d)
    assert ri.numel() > 5000
    rd = torch.randn(ri.numel(), 3, generator=torch.Generator(device="cpu").manual_seed(5)).to(dev)
    m.geometry.curvature_dirs_fn = lambda t: rd
    valid = torch.ones(n_rays, dtype=torch.bool, device=dev)
    m.zero_grad()
    out = m.forward_(rays)
    _loss(out, target, valid).backward()
    ours = {k: p.grad.detach().double().clone() for k, p in m.named_parameters() if p.grad is not None}

    c = m.config
    h = c.geometry.xyz_encoding_config
    lay = O.HashGridLayout(h.n_levels, h.n_features_per_level, h.log2_hashmap_size,
                           h.base_resolution, h.per_level_scale)
    G = dict(radius=float(c.radius), eps=float(m.geometry._finite_difference_eps), lay=lay,
             active_levels=int(m.geometry.hashgrid.mask_levels),
             n_layers=c.geometry.mlp_network_config.n_hidden_layers + 1,
             feature_dim=c.geometry.feature_dim)
    T = dict(kind="dual", n_layers=c.texture.mlp_network_config.n_hidden_layers + 1)
    Pg = {k: v.detach().double().clone().requires_grad_(v.is_floating_point())
          for k, v in m.state_dict().items()}
    march = (off.cpu().numpy(), ri.long(), t0, t1)
    # the cosine annealing ratio of global step 6000 (cos_anneal_end 20000)
    r = O.neus_render(rays.double(), Pg, G, T, march, rd.double(), float(m.cos_anneal_ratio),
                      bg.double(), training=True)
    _loss(r, target.double(), valid).backward()

    checks = []
    tk = "geometry.encoding.encoding.encoding.params"
    checks += [(tk, i) for i in torch.topk(ours[tk].abs(), 16).indices.tolist()]
    for k in ("geometry.network.layers.0.weight_v", "geometry.network.layers.0.weight_g",
              "geometry.network.layers.2.weight_v", "geometry.network.layers.4.weight_v",
              "geometry.network.layers.4.bias", "texture.network.layers.0.weight",
              "texture.network.layers.2.weight", "texture.network.layers.4.weight",
              "texture.network.layers.4.bias"):
        n = ours[k].numel()
        checks += [(k, i) for i in torch.topk(ours[k].abs().view(-1), min(4, n)).indices.tolist()]
    checks.append(("variance.variance", 0))
    rows = [(k, i, float(ours[k].view(-1)[i]), float(Pg[k].grad.view(-1)[i])) for k, i in checks]
    print("\n(param, index, fused, autograd fp64)")
    for row in rows:
        print(row)
    scale = max(abs(r_[3]) for r_ in rows)
    for k, i, a, ag in rows:
        assert abs(a - ag) <= 5e-3 * max(abs(ag), 1e-2 * scale), ("fused", k, i, a, ag)
