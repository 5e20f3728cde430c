"""CPU restatement of the Neuralangelo sparse training step, for the timed
CPU baseline of bench.py (its `cpu_baseline` leg and its `--impl reference`
arm).

ORACLE INFRASTRUCTURE ONLY: bench.py's CPU legs and tests/ use it; the
product package never imports it, and nothing here touches libangelo_gb.so.

The step is the reference's (systems/neus.py:120-206): rays with stratified
jitter -> nerfacc 0.3.3 ray marching through the occupancy grid (the C
restatement, oracle/oracle.c) -> NeuSModel.forward_ (models/neus.py:205-283):
VolumeSDF with the 6-tap FD gradient and the 6-tap curvature stencil
(models/geometry.py:195-287, reference quirks kept), the dual-colour radiance
(models/texture.py:38-64), get_alpha (models/neus.py:117-139),
render_weight_from_alpha and accumulate_along_rays -> the rgb MSE, eikonal
and curvature losses (systems/neus.py:130-159) -> backward -> AdamW
(systems/utils.py:314-325).  The arithmetic is oracle/neus_fp64.py's (the
checker; tests/test_cpu_step.py pins this module to it), in float32 and
vectorised: one gather of all levels' 8 corners per encoded point, the main
point and its FD taps in one batch, the per-ray transmittance as a padded
cumulative product, so the host cores spend their time on the step's
arithmetic rather than on Python loops.  Hash-grid cells and corner indices
come from the C restatement of tcnn's float32 grid arithmetic.

The reference runs this on tcnn / nerfacc CUDA kernels; neither has a CPU
implementation, and the reference's own Python cannot be imported where this
runs, so this restatement stands in for the reference on the host cores."""
from __future__ import annotations

import math
import time

import numpy as np
import torch
import torch.nn.functional as F

from . import cref
from . import neus_fp64 as O

_CORNER_BITS = torch.tensor([[(c >> d) & 1 for d in range(3)] for c in range(8)])


def reference_init(model_cfg, seed=0):
    """The parameters NeuSModel(model_cfg) starts from, by the reference's own
    initialisation, keyed by the reference's parameter names (float32, CPU):
    tcnn's U(-1e-4, 1e-4) table; VanillaMLP's sphere init + weight norm of the
    geometry network (models/network_utils.py:115-133) and kaiming-uniform
    texture layers with zero biases (:128-130); variance = init_val
    (models/neus.py:17-20)."""
    g = torch.Generator().manual_seed(seed)
    gc = model_cfg["geometry"]
    h = gc["xyz_encoding_config"]
    lay = O.HashGridLayout(h["n_levels"], h["n_features_per_level"], h["log2_hashmap_size"],
                           h["base_resolution"], h["per_level_scale"])
    P = {"geometry.encoding.encoding.encoding.params":
         torch.rand(lay.n_params, generator=g) * 2e-4 - 1e-4}
    m = gc["mlp_network_config"]
    n_in = 3 + lay.L * lay.F
    dims = [n_in] + [m["n_neurons"]] * m["n_hidden_layers"] + [gc["feature_dim"]]
    r = m.get("sphere_init_radius", 0.5)
    for i in range(len(dims) - 1):
        din, dout = dims[i], dims[i + 1]
        last, first = i == len(dims) - 2, i == 0
        W = torch.zeros(dout, din)
        if last:
            b = torch.full((dout,), -r)
            W.normal_(math.sqrt(math.pi) / math.sqrt(din), 1e-4, generator=g)
        else:
            b = torch.zeros(dout)
            cols = slice(0, 3) if first else slice(0, din)
            W[:, cols].normal_(0.0, math.sqrt(2) / math.sqrt(dout), generator=g)
        k = f"geometry.network.layers.{2 * i}"
        P[k + ".weight_g"] = W.norm(dim=1, keepdim=True)
        P[k + ".weight_v"] = W
        P[k + ".bias"] = b
    t = model_cfg["texture"]
    tm = t["mlp_network_config"]
    tdims = [t["input_feature_dim"] + 16] + [tm["n_neurons"]] * tm["n_hidden_layers"] + [3]
    for i in range(len(tdims) - 1):
        W = torch.empty(tdims[i + 1], tdims[i])
        torch.nn.init.kaiming_uniform_(W, nonlinearity="relu", generator=g)
        P[f"texture.network.layers.{2 * i}.weight"] = W
        P[f"texture.network.layers.{2 * i}.bias"] = torch.zeros(tdims[i + 1])
    P["variance.variance"] = torch.tensor(float(model_cfg["variance"]["init_val"]))
    return P, lay


def hash_encode(x, table, lay, active_levels):
    """tcnn HashGrid forward with the band mask (models/network_utils.py:
    56-59), all levels and corners at once: x (N,3) contracted points ->
    (N, L*F).  Differentiable in the table (one gather, one scatter-add in
    the backward)."""
    L, Fd = lay.L, lay.F
    x32 = x.detach().to(torch.float32).numpy()
    idx, _, cells = cref.hashgrid_index(x32, lay.cref_layout, with_cells=True)
    idx = torch.from_numpy(idx.astype(np.int64))                        # (N, L, 8)
    idx += torch.from_numpy(np.asarray(lay.offsets[:L], np.int64))[None, :, None]
    cells = torch.from_numpy(cells).to(x.dtype)                          # (N, L, 3)
    scales = torch.tensor(np.asarray(lay.scales[:L], np.float64), dtype=x.dtype)
    frac = x[:, None, :] * scales[None, :, None] + 0.5 - cells            # (N, L, 3)
    bits = _CORNER_BITS.to(x.dtype)                                       # (8, 3)
    f = frac[:, :, None, :]
    w = torch.where(bits.bool(), f, 1.0 - f).prod(-1)                     # (N, L, 8)
    feats = table.view(-1, Fd)[idx]                                       # (N, L, 8, F)
    enc = (w[..., None] * feats).sum(2)                                   # (N, L, F)
    act = int(active_levels)
    if act < L:
        enc = enc * (torch.arange(L) < act).to(enc.dtype)[None, :, None]
    return enc.reshape(x.shape[0], L * Fd)


def volume_sdf(points, P, G, rand_dirs):
    """VolumeSDF.forward(with_grad, with_feature, with_laplace)
    (models/geometry.py:195-287) as oracle/neus_fp64.volume_sdf computes it;
    the main point and its 6 FD taps are one batch, the 6 curvature taps a
    second.  Returns sdf (N), grad (N,3), feature (N, feature_dim+3),
    laplace (N,1)."""
    r, eps = G["radius"], G["eps"]
    lay, act = G["lay"], G["active_levels"]
    table = P["geometry.encoding.encoding.encoding.params"]
    layers = O.mlp_layers(P, "geometry.network", G["n_layers"], True)
    n = points.shape[0]
    off = torch.tensor(O._FD_OFFSETS, dtype=points.dtype) * eps

    def field(xc):
        enc = torch.cat([xc * 2.0 - 1.0, hash_encode(xc, table, lay, act)], dim=-1)
        return O.mlp(enc, layers, True)

    pts_c = O.contract(points, r)
    pd = (points[:, None, :] + off).clamp(-r, r)
    both = torch.cat([pts_c, O.contract(pd, r).reshape(-1, 3)])
    out_all = field(both)
    out = out_all[:n]
    sdf = out[:, 0]
    feature = torch.cat([out, pts_c * 2 - 1], dim=-1)
    sd = out_all[n:, 0].reshape(-1, 6)
    grad = 0.5 * (sd[:, 0::2] - sd[:, 1::2]) / eps
    rd = F.normalize(rand_dirs, dim=-1)
    normals = F.normalize(grad, dim=-1)
    tangent = torch.cross(normals, rd, dim=-1)
    shifted = pts_c + tangent * eps                   # contracted points (reference quirk)
    psd = (shifted[:, None, :] + off).clamp(-r, r)    # clamped as if world coordinates
    ssd = field(O.contract(psd, r).reshape(-1, 3))[:, 0].reshape(-1, 6)
    gs = 0.5 * (ssd[:, 0::2] - ssd[:, 1::2]) / eps
    ns = F.normalize(gs, dim=-1)
    dot = (normals * ns).sum(-1, keepdim=True)
    laplace = torch.acos(torch.clamp(dot, -1.0 + 1e-6, 1.0 - 1e-6)) / math.pi
    return sdf, grad, feature, laplace


def render_weights(alpha, offsets, early_stop_eps=1e-4):
    """render_weight_from_alpha (nerfacc 0.3.3, models/neus.py:234) as
    oracle/neus_fp64.render_weights computes it, over all rays at once:
    the samples of each ray padded to the longest ray, the exclusive
    transmittance a cumulative product along the padded rows."""
    off = torch.as_tensor(np.asarray(offsets), dtype=torch.int64)
    counts = off[1:] - off[:-1]
    R, S = counts.numel(), alpha.shape[0]
    if S == 0:
        return alpha.new_zeros(0)
    width = int(counts.max())
    ray = torch.repeat_interleave(torch.arange(R), counts)
    pos = torch.arange(S) - off[:-1][ray]
    pad = alpha.new_zeros(R, width)
    pad = pad.index_put((ray, pos), alpha)
    T = torch.cumprod(torch.cat([alpha.new_ones(R, 1), 1.0 - pad[:, :-1]], 1), 1)
    w = pad * T * (T >= early_stop_eps).to(alpha.dtype)
    return w[ray, pos]


def neus_forward(rays, P, G, T, march, rand_dirs, cos_anneal_ratio, background_color):
    """NeuSModel.forward_ (models/neus.py:205-283), training outputs, as
    oracle/neus_fp64.neus_render."""
    n_rays = rays.shape[0]
    offsets, ray_idx, t0, t1 = march
    ray_idx = torch.as_tensor(ray_idx, dtype=torch.int64)
    t0 = torch.as_tensor(t0, dtype=rays.dtype)[:, None]
    t1 = torch.as_tensor(t1, dtype=rays.dtype)[:, None]
    o, d = rays[:, 0:3], rays[:, 3:6]
    t_o, t_d = o[ray_idx], d[ray_idx]
    mid = (t0 + t1) / 2.0
    pos = t_o + t_d * mid
    sdf, grad, feat, lap = volume_sdf(pos, P, G, rand_dirs)
    normal = F.normalize(grad, p=2, dim=-1)
    alpha = O.get_alpha(sdf, normal, t_d, t1 - t0, O.inv_s(P), cos_anneal_ratio)
    rgb = O.texture(feat, t_d, normal, P, T)
    w = render_weights(alpha, offsets)
    opacity = O.accumulate(w, ray_idx, None, n_rays)
    depth = O.accumulate(w, ray_idx, mid, n_rays)
    comp_rgb = O.accumulate(w, ray_idx, rgb, n_rays)
    bg = background_color.to(comp_rgb.dtype)
    return {"comp_rgb": comp_rgb, "opacity": opacity, "depth": depth,
            "rays_valid": opacity > 0, "comp_rgb_full": comp_rgb + bg[None, :] * (1.0 - opacity),
            "sdf_samples": sdf, "sdf_grad_samples": grad, "sdf_laplace_samples": lap,
            "weights": w}


class TrainStep:
    """The full training configuration's step on the host cores: parameters
    by the reference's initialisation (the same model configuration as the
    GPU workload), the step's global step (band mask, FD eps, cosine ratio)
    and inv_s, the occupancy grid as a (res^3,) bool tensor, AdamW with the
    reference's groups.  ``step(rays, rgb)`` runs one iteration and returns
    (seconds, samples)."""

    def __init__(self, model_cfg, system_cfg, global_step, variance, occupancy, seed=0):
        self.P, self.lay = reference_init(model_cfg, seed)
        self.P["variance.variance"].fill_(float(variance))
        for v in self.P.values():
            v.requires_grad_(True)
        gc = model_cfg["geometry"]
        h = dict(gc["xyz_encoding_config"])
        self.radius = float(model_cfg["radius"])
        level = O.band_level(h, global_step)
        self.G = dict(radius=self.radius, lay=self.lay, active_levels=level,
                      n_layers=gc["mlp_network_config"]["n_hidden_layers"] + 1,
                      feature_dim=gc["feature_dim"], hg=h)
        self.G["eps"] = O.fd_eps(self.G, global_step)
        self.T = dict(kind="dual" if model_cfg["texture"]["name"] == "volume-dual-color"
                      else "radiance",
                      n_layers=model_cfg["texture"]["mlp_network_config"]["n_hidden_layers"] + 1)
        end = model_cfg.get("cos_anneal_end", 0)
        self.cos_ratio = 1.0 if end == 0 else min(1.0, global_step / end)
        self.step_size = 1.732 * 2 * self.radius / model_cfg["num_samples_per_ray"]
        self.aabb = np.array([-self.radius] * 3 + [self.radius] * 3, np.float32)
        res = round(occupancy.numel() ** (1.0 / 3.0))
        self.binary = occupancy.reshape(res, res, res).numpy().astype(np.uint8)
        loss = system_cfg["loss"]
        self.lam = (float(loss["lambda_rgb_mse"]), float(loss["lambda_eikonal"]),
                    float(loss["lambda_curvature"]))
        groups = []
        lrs = system_cfg["optimizer"]["params"]
        for name in ("geometry", "texture", "variance"):
            ps = [v for k, v in self.P.items() if k.split(".")[0] == name]
            groups.append({"params": ps, **lrs[name]})
        a = system_cfg["optimizer"]["args"]
        self.opt = torch.optim.AdamW(groups, lr=a["lr"], betas=tuple(a["betas"]), eps=a["eps"])
        self.rng = np.random.default_rng(seed + 1)

    def march(self, rays):
        o = rays[:, :3].numpy()
        d = rays[:, 3:].numpy()
        tmin, tmax = cref.ray_aabb(o, d, self.aabb)
        n = rays.shape[0]
        tmin = (tmin + self.rng.random(n, dtype=np.float32) * np.float32(self.step_size))
        _, off, ri, t0, t1, _ = cref.march(o, d, tmin.astype(np.float32), tmax, self.aabb,
                                           self.binary, self.step_size)
        return off, ri, t0, t1

    def step(self, rays, rgb, background=None):
        t_start = time.perf_counter()
        march = self.march(rays)
        n = len(march[2])
        rd = torch.randn(n, 3)
        bg = background if background is not None else torch.rand(3)
        out = neus_forward(rays, self.P, self.G, self.T, march, rd, self.cos_ratio, bg)
        loss = O.neus_losses(out, rgb, lam_rgb_mse=self.lam[0], lam_eikonal=self.lam[1],
                             lam_curvature=self.lam[2])
        self.opt.zero_grad(set_to_none=True)
        loss.backward()
        self.opt.step()
        return time.perf_counter() - t_start, n
