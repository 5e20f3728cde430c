"""Parity at the benchmark's own configuration: the Neuralangelo sparse
training step (16 levels x 2^22 entries, base 32, finest 2048; geometry
35 -> 64 -> 64 -> 65; dual-colour radiance; FD eps 1/2048 at global step
6000; inv_s = e^7; cosine-annealing ratio 0.3; 128^3 occupancy grid, step
sqrt(3) * 2 * 0.5 / 512), on the fused form the benchmark times, against the
FP64 oracle (oracle/neus_fp64.py) on the same marched samples.

Two ray sets:
* camera rays from poses on the radius-1.5 sphere through the analytic
  union scene's occupancy band (the benchmark's sampling);
* grazing rays that enter the box through a face at a shallow angle, marched
  through an all-occupied grid, so that the first samples of each ray lie
  within eps of the face and their FD taps are clamped to the box
  (models/geometry.py:230); the curvature taps clamp on every sample with a
  contracted coordinate above 1/2 (the contracted-as-world quirk,
  models/geometry.py:246,264-265).

Every forward output is compared: sdf, the FD gradient, the unit normal,
the curvature ("laplace"), per-sample weights, and per-ray colour, depth and
opacity.  Tolerances (absolute, max over every sample / ray):

* sdf, weights, colour, depth, opacity: 1e-3 (TOL);
* the FD gradient, the normal and the curvature are ill-conditioned at
  eps = 1/2048: the gradient is a difference of two SDF values divided by
  2 eps (~1000x the SDF's error; plain FP32 itself is off by ~3e-3), the
  normal divides that by |grad|, and the curvature is the angle between two
  such normals (a sign flip of a near-zero component moves it by up to 1).
  Their bound is the error of the reference's own arithmetic on the same
  inputs: tcnn (default half-precision build) uses the table in fp16 and
  returns fp16 encodings, which the reference promotes to fp32
  (models/network_utils.py:56-59, models/geometry.py:206).  The oracle run
  with the table and every encoding rounded to fp16 gives REF16, a lower
  bound on that error (tcnn also interpolates in fp16).  Bounds (FD_FACTOR =
  2): the gradient within FD_FACTOR max|sdf error| / eps (the FD difference
  of two SDF values) and its mean within FD_FACTOR x REF16's; the normal's
  max and mean within FD_FACTOR x REF16's; the curvature's mean and its
  99.9th percentile within FD_FACTOR x REF16's (+ 1e-3).

The backward (hash-table scatter-add, both MLPs' backward, the compositing
adjoint) is checked against the oracle's autograd gradient of the training
loss on the top-16 and on 64 random non-zero table entries and the top-4
plus 8 random entries of every weight tensor: relative error <= GRAD_RTOL;
the variance's within 2x the plain FP32 path's own error where that is
larger (its gradient sums sigmoid differences that cancel in fp32 below the
FP64 gate, inv_s = 2048).

A report of every error goes to $ANGELO_HEADLINE_REPORT (JSON) when set."""
import json
import math
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GLOBAL_STEP = 6000
INV_S_VARIANCE = 0.7        # inv_s = exp(7)
REPORT = {}

# max absolute error against FP64 of each forward output
TOL = {"sdf": 1e-3, "grad": 1e-3, "normal": 1e-3, "laplace": 1e-3, "weights": 1e-3,
       "rgb": 1e-3, "depth": 1e-3, "opacity": 1e-3}


def _write():
    path = os.environ.get("ANGELO_HEADLINE_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _set_grid(m, occ):
    from angelo_gb.checkpoint import pack_bits
    dev = m.occupancy_grid.bits.device
    m.occupancy_grid.bits.copy_(pack_bits(occ.reshape(-1).cpu()).to(dev))
    m.occupancy_grid.occs.copy_(occ.reshape(-1).float().to(dev))


@pytest.fixture(scope="module")
def models_(dev):
    """The fused model at the benchmark's state and a plain copy of it.  The
    table and the first layer's hash columns get values that make every
    level matter (U(-0.05, 0.05) and N(0, 0.05^2))."""
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    fused = models.make("neus", workloads.model_config("full", fused=True)).to(dev)
    plain = models.make("neus", workloads.model_config("full", fused=False)).to(dev)
    with torch.no_grad():
        g = torch.Generator(device="cpu").manual_seed(7)
        p = fused.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=g) * 0.1 - 0.05).to(dev))
        wv = fused.geometry.network.layers[0].weight_v
        wv[:, 3:].copy_((torch.randn(wv[:, 3:].shape, generator=g) * 0.05).to(dev))
        fused.variance.variance.fill_(INV_S_VARIANCE)
    plain.load_state_dict(fused.state_dict())
    for m in (fused, plain):
        m.update_step(0, GLOBAL_STEP)
        m.train()
        m.randomized = False
    return fused, plain


def _camera_rays(dev, n=256, seed=3):
    from angelo_gb.scenes import pixel_directions, rays_from, sphere_poses
    g = np.random.default_rng(seed)
    poses = sphere_poses(8, 1.5, seed).float().to(dev)
    dirs = pixel_directions(1600, 1200, 40.0, device=dev).reshape(-1, 3)
    pix = torch.from_numpy(g.integers(0, dirs.shape[0], n)).to(dev)
    cam = torch.from_numpy(g.integers(0, 8, n)).to(dev)
    return rays_from(dirs[pix], poses[cam]).float().contiguous()


def _grazing_rays(dev, n=32, seed=4):
    """Rays entering the [-0.5, 0.5]^3 box through one of its six faces at
    about 8 degrees to the face: the first sample of each lies within eps of
    that face."""
    g = np.random.default_rng(seed)
    rays = []
    for i in range(n):
        axis, sign = i % 3, (-1.0) ** (i // 3)
        entry = g.uniform(-0.3, 0.3, 3)
        entry[axis] = 0.5 * sign
        tang = g.normal(size=3)
        tang[axis] = 0.0
        tang /= np.linalg.norm(tang)
        d = tang.copy()
        d[axis] = -sign * 0.14                     # pointing into the box
        d /= np.linalg.norm(d)
        o = entry - d * 0.6
        rays.append(np.concatenate([o, d]))
    return torch.tensor(np.array(rays), dtype=torch.float32, device=dev)


def _oracle(m, rays, march, rd, bg):
    from oracle import neus_fp64 as O
    c = m.config
    h = c.geometry.xyz_encoding_config
    lay = O.HashGridLayout(h.n_levels, h.n_features_per_level, h.log2_hashmap_size,
                           h.base_resolution, h.per_level_scale)
    G = dict(radius=float(c.radius), eps=float(m.geometry._finite_difference_eps), lay=lay,
             active_levels=int(m.geometry.hashgrid.mask_levels),
             n_layers=c.geometry.mlp_network_config.n_hidden_layers + 1,
             feature_dim=c.geometry.feature_dim)
    T = dict(kind="dual", n_layers=c.texture.mlp_network_config.n_hidden_layers + 1)
    return G, T, O


def _err(a, b):
    d = (a.double().reshape(b.shape) - b.double()).abs()
    return float(d.max()) if d.numel() else 0.0


def _mean_err(a, b):
    d = (a.double().reshape(b.shape) - b.double()).abs()
    return float(d.mean()) if d.numel() else 0.0


def _p999_err(a, b):
    d = (a.double().reshape(b.shape) - b.double()).abs().reshape(-1)
    return float(torch.quantile(d.float().cpu(), 0.999)) if d.numel() else 0.0


FD_FACTOR = 2.0


ILL_CONDITIONED = ("grad", "normal", "laplace")


def _render_fp16_encodings(O, *args):
    """The oracle's render with the hash table and every encoding rounded to
    fp16, as tcnn's half-precision HashGrid computes them."""
    orig = O.hash_encode

    def enc16(x, table, lay, active_levels=None):
        return orig(x, table.half().double(), lay, active_levels).half().double()

    O.hash_encode = enc16
    try:
        return O.neus_render(*args, training=True)
    finally:
        O.hash_encode = orig


def _forward_errors(dev, models_, rays, occ, label):
    from torch.nn.functional import normalize
    fused, plain = models_
    for m in (fused, plain):
        _set_grid(m, occ)
    assert abs(float(fused.geometry._finite_difference_eps) - 1.0 / 2048) < 1e-9
    assert int(fused.geometry.hashgrid.mask_levels) == 16
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, off = fused.march_rays(o, d)
    n = ri.numel()
    assert n > 2000, n
    rd = torch.randn(n, 3, generator=torch.Generator(device="cpu").manual_seed(5)).to(dev)
    bg = torch.tensor([0.3, 0.6, 0.9], device=dev)
    outs = {}
    for name, m in (("fused", fused), ("plain_fp32", plain)):
        m.background_color = bg
        m.geometry.curvature_dirs_fn = lambda t: rd
        with torch.no_grad():
            outs[name] = m.forward_(rays)
        assert int(outs[name]["num_samples_full"].sum()) == n
    G, T, O = _oracle(fused, rays, None, rd, bg)
    P = {k: v.detach().double() for k, v in fused.state_dict().items()}
    args = (rays.double(), P, G, T, (off.cpu().numpy(), ri.long(), t0, t1), rd.double(),
            float(fused.cos_anneal_ratio), bg.double())
    with torch.no_grad():
        ref = O.neus_render(*args, training=True)
        outs["ref16"] = _render_fp16_encodings(O, *args)
    rn = normalize(ref["sdf_grad_samples"], dim=-1)
    rows = {}
    for name, r in outs.items():
        pairs = {
            "sdf": (r["sdf_samples"], ref["sdf_samples"]),
            "grad": (r["sdf_grad_samples"], ref["sdf_grad_samples"]),
            "normal": (normalize(r["sdf_grad_samples"].double(), dim=-1), rn),
            "laplace": (r["sdf_laplace_samples"], ref["sdf_laplace_samples"]),
            "weights": (r["weights"], ref["weights"]),
            "rgb": (r["comp_rgb_full"], ref["comp_rgb_full"]),
            "depth": (r["depth"], ref["depth"]),
            "opacity": (r["opacity"], ref["opacity"]),
        }
        rows[name] = {k: _err(a, b) for k, (a, b) in pairs.items()}
        rows[name + "_mean"] = {k: _mean_err(a, b) for k, (a, b) in pairs.items()}
        rows[name + "_p999"] = {k: _p999_err(a, b) for k, (a, b) in pairs.items()
                                if k in ILL_CONDITIONED}
    # how many samples had a clamped FD tap (the boundary path)
    pos = (o[ri.long()] + d[ri.long()] * ((t0 + t1) * 0.5)[:, None])
    clamped = int(((pos.abs() + 1.0 / 2048) > 0.5).any(-1).sum())
    rows["samples"], rows["fd_clamped_samples"] = n, clamped
    rows["grad_scale"] = float(ref["sdf_grad_samples"].abs().max())
    rows["eps"] = float(G["eps"])
    REPORT[label] = rows
    _write()
    return rows


def _occupancy(dev, kind):
    if kind == "all":
        return torch.ones(128 ** 3, dtype=torch.bool)
    from angelo_gb import scenes
    return scenes.analytic_occupancy(scenes.UnionScene(), 128, device=dev).reshape(-1).cpu()


def _check(rows):
    f, fm, fp = rows["fused"], rows["fused_mean"], rows["fused_p999"]
    r, rm, rp = rows["ref16"], rows["ref16_mean"], rows["ref16_p999"]
    for k, tol in TOL.items():
        if k not in ILL_CONDITIONED:
            assert f[k] <= tol, (k, f[k], tol, rows)
    # the FD difference of two SDF values, each off by about max|sdf err|
    assert f["grad"] <= FD_FACTOR * f["sdf"] / rows["eps"], rows
    for k in ILL_CONDITIONED:
        assert fm[k] <= max(TOL[k], FD_FACTOR * rm[k]), (k, rows)
    assert f["normal"] <= max(TOL["normal"], FD_FACTOR * r["normal"]), rows
    assert fp["laplace"] <= FD_FACTOR * rp["laplace"] + 1e-3, rows


def test_headline_forward_camera_rays(dev, models_):
    rows = _forward_errors(dev, models_, _camera_rays(dev), _occupancy(dev, "band"), "camera_rays")
    _check(rows)


def test_headline_forward_grazing_rays(dev, models_):
    rows = _forward_errors(dev, models_, _grazing_rays(dev), _occupancy(dev, "all"), "grazing_rays")
    assert rows["fd_clamped_samples"] >= 16, rows
    _check(rows)


def _loss(out, target):
    valid = (out["rays_valid_full"] if "rays_valid_full" in out else out["rays_valid"])[:, 0]
    l_rgb = ((out["comp_rgb_full"][valid] - target[valid]) ** 2).mean() * 10.0
    l_eik = ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean() * 0.1
    l_curv = out["sdf_laplace_samples"].abs().mean() * 5e-4
    return l_rgb + l_eik + l_curv


GRAD_RTOL = 5e-3


def test_headline_backward_matches_fp64(dev, models_):
    """The fused backward of the training loss at the benchmark's
    configuration (camera rays through the occupancy band, where the FD taps
    of samples on the box faces are clamped too) against the FP64 autograd
    gradient of the same loss on the same samples.  Relative error per
    entry, against max(|g|, 1e-2 * the largest |g| of the checked set)."""
    fused, plain = models_
    _set_grid(fused, _occupancy(dev, "band"))
    _set_grid(plain, _occupancy(dev, "band"))
    rays = torch.cat([_camera_rays(dev, 64, seed=8), _grazing_rays(dev, 8, seed=9)])
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, off = fused.march_rays(o, d)
    n = ri.numel()
    rd = torch.randn(n, 3, generator=torch.Generator(device="cpu").manual_seed(6)).to(dev)
    bg = torch.tensor([0.3, 0.6, 0.9], device=dev)
    target = torch.from_numpy(np.random.default_rng(2).uniform(0, 1, (rays.shape[0], 3))
                              .astype(np.float32)).to(dev)
    grads = {}
    for name, m in (("fused", fused), ("plain_fp32", plain)):
        m.background_color = bg
        m.geometry.curvature_dirs_fn = lambda t: rd
        m.zero_grad()
        out = m.forward_(rays)
        _loss(out, target).backward()
        grads[name] = {k: p.grad.detach().double().clone() for k, p in m.named_parameters()
                       if p.grad is not None}
        m.zero_grad()
    ours = grads["fused"]
    G, T, O = _oracle(fused, rays, None, rd, bg)
    Pg = {k: v.detach().double().clone().requires_grad_(v.is_floating_point())
          for k, v in fused.state_dict().items()}
    r = O.neus_render(rays.double(), Pg, G, T, (off.cpu().numpy(), ri.long(), t0, t1), rd.double(),
                      float(fused.cos_anneal_ratio), bg.double(), training=True)
    _loss(r, target.double()).backward()

    gsel = torch.Generator(device="cpu").manual_seed(11)
    checks = []
    tk = "geometry.encoding.encoding.encoding.params"
    ref_t = Pg[tk].grad.view(-1)
    checks += [(tk, i) for i in torch.topk(ref_t.abs(), 16).indices.tolist()]
    nz = torch.nonzero(ref_t).view(-1).cpu()
    checks += [(tk, int(i)) for i in nz[torch.randperm(nz.numel(), generator=gsel)[:64]]]
    for k in ours:
        if k == tk:
            continue
        g = Pg[k].grad.view(-1)
        checks += [(k, i) for i in torch.topk(g.abs(), min(4, g.numel())).indices.tolist()]
        checks += [(k, int(i)) for i in torch.randperm(g.numel(), generator=gsel)[:8]]
    pl = grads["plain_fp32"]
    rows = [(k, i, float(ours[k].view(-1)[i]), float(pl[k].view(-1)[i]), float(Pg[k].grad.view(-1)[i]))
            for k, i in checks]
    scale = {}
    for k, _, _, _, ag in rows:
        scale[k] = max(scale.get(k, 0.0), abs(ag))
    worst, worst_plain = {}, {}
    for k, i, a, b, ag in rows:
        den = max(abs(ag), 1e-2 * scale[k], 1e-30)
        worst[k] = max(worst.get(k, 0.0), abs(a - ag) / den)
        worst_plain[k] = max(worst_plain.get(k, 0.0), abs(b - ag) / den)
    REPORT["backward"] = {"samples": n, "checked": len(rows), "max_rel_err": worst,
                          "plain_fp32_max_rel_err": worst_plain}
    _write()
    for k, e in worst.items():
        # the plain path's geometry gradients carry the reference formulation's
        # 1e12-scaled cancelling terms (coincident curvature taps), so only
        # the variance's bound refers to it
        bound = max(GRAD_RTOL, 2.0 * worst_plain[k]) if k == "variance.variance" else GRAD_RTOL
        assert e <= bound, (k, e, worst, worst_plain)
