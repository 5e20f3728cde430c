"""FP64 PyTorch restatement of Instant-angelo's NeuS / Neuralangelo hot path.

TEST INFRASTRUCTURE ONLY (the oracle): ``tests/``, ``__graft_entry__.smoke`` and
the CPU-baseline leg of ``bench.py`` call it as the checker.  The product package
never imports it.

Everything is a plain function of a parameter dict whose keys follow the
reference module tree (``geometry.encoding.encoding.encoding.params`` is the tcnn
flat parameter vector, ``geometry.network.layers.0.weight_v`` etc.), so one dict
feeds the reference's own modules (through the stub harness in
``oracle/ref_harness.py``), this oracle and the CUDA path alike.

Hash-grid cells and corner indices come from the C restatement (float32
arithmetic exactly as tcnn's kernel performs it, see ``oracle.c``); trilinear
weights and everything downstream are float64 and differentiable, so
``torch.autograd`` on this module is the gradient reference.  The float64
arithmetic runs on the device of its inputs (the precision study runs it on
the GPU); the cells are always computed on the host.
"""
from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn.functional as F

from . import cref

# ------------------------------------------------------------------ encodings


class HashGridLayout:
    """tcnn HashGrid layout (models/network_utils.py:40-54 builds it)."""

    def __init__(self, n_levels, n_features_per_level, log2_hashmap_size, base_resolution,
                 per_level_scale):
        self.L = int(n_levels)
        self.F = int(n_features_per_level)
        self.log2T = int(log2_hashmap_size)
        self.base = int(base_resolution)
        self.b = float(per_level_scale)
        self.offsets, self.res, self.scales = cref.hashgrid_layout(self.L, self.log2T, self.base,
                                                                   self.b)
        self.n_entries = int(self.offsets[-1])
        self.n_params = self.n_entries * self.F

    @property
    def cref_layout(self):
        return (self.offsets, self.res, self.scales)


def hash_encode(x, table, lay: HashGridLayout, active_levels=None):
    """tcnn HashGrid forward ``enc`` followed by the band mask ``enc * mask``
    (models/network_utils.py:56-59).  x: (N,3) float64 in contracted [0,1]
    coordinates (differentiable); table: (n_entries*F,) float64.
    Returns (N, L*F) float64."""
    L, Fd = lay.L, lay.F
    act = L if active_levels is None else int(active_levels)
    x32 = x.detach().to(torch.float32).cpu().numpy()
    idx, _, cells = cref.hashgrid_index(x32, lay.cref_layout, with_cells=True)
    idx = torch.from_numpy(idx.astype(np.int64)).to(x.device)
    cells = torch.from_numpy(cells.astype(np.float64)).to(device=x.device, dtype=x.dtype)
    tab = table.view(-1, Fd)
    outs = []
    for l in range(L):
        if l >= act:
            outs.append(torch.zeros(x.shape[0], Fd, dtype=x.dtype, device=x.device))
            continue
        s = float(lay.scales[l])
        frac = x * s + 0.5 - cells[:, l, :]              # (N,3), float64, d/dx = scale
        acc = 0.0
        for c in range(8):
            w = 1.0
            for d in range(3):
                w = w * (frac[:, d] if (c >> d) & 1 else 1.0 - frac[:, d])
            e = idx[:, l, c] + int(lay.offsets[l])
            acc = acc + w[:, None] * tab[e]
        outs.append(acc)
    return torch.cat(outs, dim=-1)


def composite_encode(x, table, lay, active_levels=None, include_xyz=True):
    """CompositeEncoding with include_xyz (models/network_utils.py:69-80,92):
    cat([x*2-1, enc(x)])."""
    enc = hash_encode(x, table, lay, active_levels)
    return torch.cat([x * 2.0 - 1.0, enc], dim=-1) if include_xyz else enc


_SH_C = None


def sh4(d01):
    """tcnn SphericalHarmonics degree 4 of a direction given in [0,1]^3
    (models/texture.py:24-25), differentiable float64."""
    x = d01[:, 0] * 2 - 1
    y = d01[:, 1] * 2 - 1
    z = d01[:, 2] * 2 - 1
    sp = math.sqrt(math.pi)
    c0, c1 = 1 / (2 * sp), math.sqrt(3) / (2 * sp)
    c2a, c2b, c2c = math.sqrt(15) / (2 * sp), math.sqrt(5) / (4 * sp), math.sqrt(15) / (4 * sp)
    c3a, c3b, c3c = math.sqrt(70) / (8 * sp), math.sqrt(105) / (2 * sp), math.sqrt(42) / (8 * sp)
    c3d, c3e = math.sqrt(7) / (4 * sp), math.sqrt(105) / (4 * sp)
    xy, xz, yz, x2, y2, z2 = x * y, x * z, y * z, x * x, y * y, z * z
    cols = [torch.full_like(x, c0), -c1 * y, c1 * z, -c1 * x, c2a * xy, -c2a * yz,
            c2b * (3 * z2 - 1), -c2a * xz, c2c * (x2 - y2), c3a * y * (-3 * x2 + y2),
            c3b * xy * z, c3c * y * (1 - 5 * z2), c3d * z * (5 * z2 - 3),
            c3c * x * (1 - 5 * z2), c3e * z * (x2 - y2), c3a * x * (-x2 + 3 * y2)]
    return torch.stack(cols, dim=-1)


# ----------------------------------------------------------------------- MLPs


def mlp_layers(P, prefix, n_layers, weight_norm):
    """Effective (W, b) of each nn.Linear of a VanillaMLP
    (models/network_utils.py:96-133).  weight_norm: W = g * v / ||v||_row."""
    out = []
    for i in range(n_layers):
        k = f"{prefix}.layers.{2 * i}"
        if weight_norm:
            v, g = P[k + ".weight_v"], P[k + ".weight_g"]
            W = g * v / v.norm(dim=1, keepdim=True)
        else:
            W = P[k + ".weight"]
        out.append((W, P[k + ".bias"]))
    return out


def mlp(x, layers, sphere_init):
    """VanillaMLP forward: Linear -> act -> ... -> Linear, output activation
    none.  act = Softplus(beta=100) when sphere_init else ReLU
    (models/network_utils.py:136-140)."""
    h = x
    for i, (W, b) in enumerate(layers):
        h = F.linear(h, W, b)
        if i < len(layers) - 1:
            h = F.softplus(h, beta=100) if sphere_init else F.relu(h)
    return h


# ------------------------------------------------------------------- geometry


def contract(x, r):
    """scale_anything(x, (-r, r), (0, 1)) (models/utils.py:109-114,
    models/geometry.py:21)."""
    return (x - (-r)) / (r - (-r)) * (1 - 0) + 0


_FD_OFFSETS = [[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]]


def volume_sdf(points, P, G, rand_dirs=None, with_grad=True, with_feature=True,
               with_laplace=False):
    """VolumeSDF.forward with grad_type='finite_difference'
    (models/geometry.py:195-287).  G holds the geometry config:
    radius, eps, lay (HashGridLayout), active_levels, n_layers, feature_dim.
    rand_dirs replaces torch.randn_like at models/geometry.py:238."""
    r, eps = G["radius"], G["eps"]
    lay, act = G["lay"], G["active_levels"]
    table = P["geometry.encoding.encoding.encoding.params"]
    layers = mlp_layers(P, "geometry.network", G["n_layers"], True)

    def field(xc):
        return mlp(composite_encode(xc, table, lay, act), layers, True)

    pts_c = contract(points, r)
    out = field(pts_c)
    sdf = out[:, 0]
    feature = torch.cat([out, pts_c * 2 - 1], dim=-1)
    rv = [sdf]
    grad = None
    if with_grad:
        off = torch.tensor(_FD_OFFSETS, dtype=points.dtype, device=points.device) * eps
        pd = (points[:, None, :] + off).clamp(-r, r)
        sd = field(contract(pd, r).reshape(-1, 3))[:, 0].reshape(-1, 6)
        grad = 0.5 * (sd[:, 0::2] - sd[:, 1::2]) / eps
        rv.append(grad)
    if with_feature:
        rv.append(feature)
    if with_laplace:
        rd = F.normalize(rand_dirs, dim=-1)
        normals = F.normalize(grad, dim=-1)
        tangent = torch.cross(normals, rd, dim=-1)
        shifted = pts_c + tangent * eps                 # contracted points (reference quirk)
        off = torch.tensor(_FD_OFFSETS, dtype=points.dtype, device=points.device) * eps
        psd = (shifted[:, None, :] + off).clamp(-r, r)  # clamped as if world coordinates
        ssd = field(contract(psd, r).reshape(-1, 3))[:, 0].reshape(-1, 6)
        gs = 0.5 * (ssd[:, 0::2] - ssd[:, 1::2]) / eps
        ns = F.normalize(gs, dim=-1)
        dot = (normals * ns).sum(-1, keepdim=True)
        angle = torch.acos(torch.clamp(dot, -1.0 + 1e-6, 1.0 - 1e-6))
        rv.append(angle / math.pi)
    return rv


def fd_eps(G, global_step):
    """finite_difference_eps='progressive' (models/geometry.py:301-312)."""
    h = G["hg"]
    level = min(h["start_level"] + max(global_step - h["start_step"], 0) // h["update_steps"],
                h["n_levels"])
    grid_res = h["base_resolution"] * h["per_level_scale"] ** (level - 1)
    return 2 * G["radius"] / grid_res


def band_level(h, global_step):
    """ProgressiveBandHashGrid.update_step (models/network_utils.py:61-66)."""
    return min(h["start_level"] + max(global_step - h["start_step"], 0) // h["update_steps"],
               h["n_levels"])


# -------------------------------------------------------------------- texture


def texture(features, dirs, normal, P, T):
    """VolumeRadiance (models/texture.py:23-30) when T['kind']=='radiance',
    VolumeDualColor (models/texture.py:50-58) when 'dual'."""
    d01 = (dirs + 1.0) / 2.0
    emb = sh4(d01)
    inp = torch.cat([features, emb, normal], dim=-1)
    layers = mlp_layers(P, "texture.network", T["n_layers"], False)
    color = mlp(inp, layers, False)
    if T["kind"] == "dual":
        return torch.sigmoid(color) + torch.sigmoid(features[..., 1:4])
    return torch.sigmoid(color)


def ide(xyz, kappa_inv, deg):
    """Integrated directional encoding (models/utils.py:209-273; Ref-NeRF eq.
    6-8): for l = 2^i (i < deg), m = 0..l, (x + i y)^m N_lm Q_l^m(z)
    exp(-l(l+1)/2 kappa_inv), real parts then imaginary parts.  Q_l^m =
    P_l^m / (1 - z^2)^(m/2) (Condon-Shortley phase) by the recurrence in l:
    Q_m^m = (-1)^m (2m-1)!!, Q_{m+1}^m = (2m+1) z Q_m^m,
    (l - m) Q_l^m = (2l - 1) z Q_{l-1}^m - (l + m - 1) Q_{l-2}^m."""
    x, y, z = xyz[..., 0:1], xyz[..., 1:2], xyz[..., 2:3]
    w = torch.complex(x, y)
    re, im = [], []
    for i in range(deg):
        l = 2 ** i
        for m in range(l + 1):
            q_prev, q = None, torch.full_like(z, (-1.0) ** m * float(np.prod(np.arange(2 * m - 1, 0, -2))))
            for ll in range(m + 1, l + 1):
                nxt = ((2 * ll - 1) * z * q - ((ll + m - 1) * q_prev if q_prev is not None else 0.0)) / (ll - m)
                q_prev, q = q, nxt
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - m) / math.factorial(l + m))
            val = w ** m * (norm * q * torch.exp(-0.5 * l * (l + 1) * kappa_inv))
            re.append(val.real)
            im.append(val.imag)
    return torch.cat(re + im, dim=-1)


def texture_v3(features, viewdirs, normals, P, T):
    """VolumeDualColorV3 (models/texture.py:127-146): camera and reflected
    branches blended by a weight MLP."""
    emb = sh4((viewdirs + 1.0) / 2.0)
    vdotn = (-viewdirs * normals).sum(-1, keepdim=True)
    ref = 2 * vdotn * normals + viewdirs
    if T.get("ide_degree"):
        # reflection branch on the IDE of (r + 1) / 2 with roughness
        # sigmoid(feature 5), the reference's use_ide form (models/texture.py:91-95)
        remb = ide((ref + 1.0) / 2.0, torch.sigmoid(features[..., 5:6]), T["ide_degree"])
    else:
        remb = sh4((ref + 1.0) / 2.0)
    inp = torch.cat([features, normals], dim=-1)
    wl = mlp_layers(P, "texture.weight_network", T["n_weight_layers"], False)
    wgt = mlp(inp, wl, False)
    if T.get("weight_activation") == "sigmoid":
        wgt = torch.sigmoid(wgt)
    cl = mlp_layers(P, "texture.cam_network", T["n_layers"], False)
    rl = mlp_layers(P, "texture.ref_network", T["n_layers"], False)
    cam = mlp(torch.cat([inp, emb], -1), cl, False)
    refc = mlp(torch.cat([inp, remb], -1), rl, False)
    return wgt * torch.sigmoid(refc) + (1 - wgt) * torch.sigmoid(cam)


# ------------------------------------------------------------------ renderer


def inv_s(P):
    """VarianceNetwork.inv_s = exp(10 * variance) (models/neus.py:27-32)."""
    return torch.exp(P["variance.variance"] * 10.0)


def get_alpha(sdf, normal, dirs, dists, s, cos_anneal_ratio):
    """NeuSModel.get_alpha (models/neus.py:117-139)."""
    s = s.clip(1e-6, 1e6)
    true_cos = (dirs * normal).sum(-1, keepdim=True)
    iter_cos = -(F.relu(-true_cos * 0.5 + 0.5) * (1.0 - cos_anneal_ratio) +
                 F.relu(-true_cos) * cos_anneal_ratio)
    nxt = sdf[..., None] + iter_cos * dists.reshape(-1, 1) * 0.5
    prv = sdf[..., None] - iter_cos * dists.reshape(-1, 1) * 0.5
    pc = torch.sigmoid(prv * s)
    nc = torch.sigmoid(nxt * s)
    return ((pc - nc + 1e-5) / (pc + 1e-5)).view(-1).clip(0.0, 1.0)


def render_weights(alpha, offsets, early_stop_eps=1e-4):
    """render_weight_from_alpha (nerfacc 0.3.3, models/neus.py:234): per ray,
    w_j = alpha_j * prod_{k<j}(1 - alpha_k), zero once the transmittance has
    dropped below early_stop_eps.  Differentiable float64."""
    n = alpha.shape[0]
    out = torch.zeros(n, dtype=alpha.dtype, device=alpha.device)
    ws = []
    for r in range(len(offsets) - 1):
        a = alpha[offsets[r]:offsets[r + 1]]
        if a.numel() == 0:
            continue
        T = torch.cumprod(torch.cat([torch.ones(1, dtype=a.dtype, device=a.device), 1 - a[:-1]]), 0)
        ws.append(a * T * (T >= early_stop_eps).to(a.dtype))
    if ws:
        out = torch.cat(ws)
    return out


def accumulate(w, ray_indices, values, n_rays):
    """accumulate_along_rays (nerfacc 0.3.3, models/neus.py:235-240)."""
    src = w[:, None] if values is None else w[:, None] * values
    out = torch.zeros(n_rays, src.shape[-1], dtype=src.dtype, device=src.device)
    return out.index_add(0, ray_indices, src)


def neus_render(rays, P, G, T, march, rand_dirs, cos_anneal_ratio, background_color,
                training=True):
    """NeuSModel.forward_ (models/neus.py:205-283) without the learned
    background.  ``march`` = (offsets, ray_indices, t_starts, t_ends) from the
    nerfacc restatement (integers and float32 t); everything else float64."""
    n_rays = rays.shape[0]
    offsets, ray_idx, t0, t1 = march
    ray_idx = torch.as_tensor(ray_idx, dtype=torch.int64, device=rays.device)
    t0 = torch.as_tensor(t0, dtype=rays.dtype, device=rays.device)[:, None]
    t1 = torch.as_tensor(t1, dtype=rays.dtype, device=rays.device)[:, None]
    o, d = rays[:, 0:3], rays[:, 3:6]
    t_o, t_d = o[ray_idx], d[ray_idx]
    mid = (t0 + t1) / 2.0
    pos = t_o + t_d * mid
    dists = t1 - t0
    sdf, grad, feat, lap = volume_sdf(pos, P, G, rand_dirs, True, True, True)
    normal = F.normalize(grad, p=2, dim=-1)
    alpha = get_alpha(sdf, normal, t_d, dists, inv_s(P), cos_anneal_ratio)
    if T["kind"] == "v3":
        rgb = texture_v3(feat, t_d, normal, P, T)
    else:
        rgb = texture(feat, t_d, normal, P, T)
    w = render_weights(alpha, list(np.asarray(offsets)))
    opacity = accumulate(w, ray_idx, None, n_rays)
    depth = accumulate(w, ray_idx, mid, n_rays)
    comp_rgb = accumulate(w, ray_idx, rgb, n_rays)
    fg = opacity > 0.1
    cn = F.normalize(accumulate(w, ray_idx, normal, n_rays), p=2, dim=-1)
    cn = torch.where(fg, cn, torch.zeros_like(cn))
    bg = background_color.to(comp_rgb.dtype)
    out = {
        "comp_rgb": comp_rgb, "comp_normal": cn, "opacity": opacity, "depth": depth,
        "rays_valid": opacity > 0, "num_samples": torch.tensor([len(t0)], dtype=torch.int32),
        "comp_rgb_full": comp_rgb + bg[None, :] * (1.0 - opacity),
    }
    if training:
        out.update({"sdf_samples": sdf, "sdf_grad_samples": grad, "weights": w,
                    "points": mid.view(-1), "intervals": dists.view(-1), "ray_indices": ray_idx,
                    "sdf_laplace_samples": lap, "alpha": alpha, "rgb_samples": rgb})
    return out


# ---------------------------------------------------------- learned background


def contract_unbounded(x, r):
    """UN_BOUNDED_SPHERE contraction (models/geometry.py:22-28)."""
    x = contract(x, r) * 2 - 1
    mag = x.norm(dim=-1, keepdim=True)
    x = torch.where(mag > 1, (2 - 1 / mag) * (x / mag), x)
    return x / 4 + 0.5


def volume_density(points, P, B):
    """VolumeDensity.forward (models/geometry.py:162-170) with the sparse
    configs' trunc_exp density: B holds radius, lay, active_levels, n_layers,
    density_bias.  Returns (density, feature)."""
    x = contract_unbounded(points, B["radius"])
    pre = "geometry_bg.encoding_with_network"
    enc = composite_encode(x, P[pre + ".encoding.encoding.encoding.params"], B["lay"],
                           B["active_levels"])
    out = mlp(enc, mlp_layers(P, pre + ".network", B["n_layers"], False), False)
    return torch.exp(out[:, 0] + B["density_bias"]), out


def texture_bg(features, dirs, P, n_layers):
    """VolumeRadiance without normals (models/texture.py:23-30, the
    background's texture): sigmoid(MLP(cat(feature, SH4((d+1)/2))))."""
    inp = torch.cat([features, sh4((dirs + 1.0) / 2.0)], dim=-1)
    return torch.sigmoid(mlp(inp, mlp_layers(P, "texture_bg.network", n_layers, False), False))


def density_weights(t0, t1, sigma, offsets):
    """render_weight_from_density (nerfacc 0.3.3, models/neus.py:171): per ray
    w_j = (1 - exp(-tau_j)) exp(-sum_{k<j} tau_k), tau = sigma (t1 - t0)."""
    tau = sigma * (t1 - t0)
    ws = []
    for r in range(len(offsets) - 1):
        t = tau[offsets[r]:offsets[r + 1]]
        if t.numel() == 0:
            continue
        before = torch.cat([torch.zeros(1, dtype=t.dtype, device=t.device), torch.cumsum(t, 0)[:-1]])
        ws.append((1 - torch.exp(-t)) * torch.exp(-before))
    return torch.cat(ws) if ws else torch.zeros_like(tau)


def render_bg(rays, P, B, n_layers_tex, march, background_color):
    """NeuSModel.forward_bg_ (models/neus.py:141-203) on given samples
    ``march`` = (offsets, ray_indices, t_starts, t_ends) after the visibility
    test; float64.  Returns comp_rgb (background colour blended), opacity,
    depth."""
    n_rays = rays.shape[0]
    offsets, ray_idx, t0, t1 = march
    ray_idx = torch.as_tensor(ray_idx, dtype=torch.int64, device=rays.device)
    t0 = torch.as_tensor(t0, dtype=rays.dtype, device=rays.device)
    t1 = torch.as_tensor(t1, dtype=rays.dtype, device=rays.device)
    o, d = rays[:, 0:3], rays[:, 3:6]
    mid = (t0 + t1) / 2.0
    pos = o[ray_idx] + d[ray_idx] * mid[:, None]
    density, feat = volume_density(pos, P, B)
    rgb = texture_bg(feat, d[ray_idx], P, n_layers_tex)
    w = density_weights(t0, t1, density, list(np.asarray(offsets)))
    opacity = accumulate(w, ray_idx, None, n_rays)
    depth = accumulate(w, ray_idx, mid[:, None], n_rays)
    comp = accumulate(w, ray_idx, rgb, n_rays)
    comp = comp + background_color.to(comp.dtype)[None, :] * (1.0 - opacity)
    return {"comp_rgb": comp, "opacity": opacity, "depth": depth, "weights": w}


def neus_loss_terms(out, rgb_target, lam_rgb_mse=10.0, lam_eikonal=0.1, lam_curvature=5e-4):
    """The hot-path loss seeds of NeuSSystem.training_step
    (systems/neus.py:130-159), weighted: (rgb MSE on valid rays + eikonal,
    curvature)."""
    valid = out["rays_valid"][:, 0]
    l_rgb = F.mse_loss(out["comp_rgb_full"][valid], rgb_target[valid])
    l_eik = ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean()
    l_curv = out["sdf_laplace_samples"].abs().mean()
    return l_rgb * lam_rgb_mse + l_eik * lam_eikonal, l_curv * lam_curvature


def neus_losses(out, rgb_target, **kw):
    a, b = neus_loss_terms(out, rgb_target, **kw)
    return a + b
