"""The hot-path part of NeuSSystem.training_step (systems/neus.py:120-206):
loss seeds (rgb MSE on valid rays, eikonal, curvature), dynamic ray-count
update (:126-128) and the AdamW step of the reference's optimizer config
(systems/utils.py:314-325).  Data loading, logging, validation and the
Lightning loop are outside the path."""
from __future__ import annotations

import torch

from .config import scheduled_value, to_config
from .optim import AdamW


def psnr(inputs, targets, valid_mask=None):
    """PSNR of systems/criterions.py:40-53 (reduction 'mean'):
    -10 log10(mean((inputs - targets)^2)) over the valid entries."""
    value = (inputs - targets) ** 2
    if valid_mask is not None:
        value = value[valid_mask]
    return -10.0 * torch.log10(torch.mean(value))


def loss_terms(out, rgb, eikonal_weight=0.1, curvature_weight=5e-4, rgb_mse_weight=10.0):
    """Weighted loss terms of systems/neus.py:130-159 (the ones the hot path
    seeds).  Returns (total, dict of unweighted terms)."""
    # F.mse_loss over the valid rays (systems/neus.py:130), as a masked
    # mean: no device-to-host read of the valid count inside the step
    valid = out["rays_valid_full"][..., 0:1].to(rgb.dtype)
    l_rgb = (((out["comp_rgb_full"] - rgb) ** 2) * valid).sum() / (valid.sum() * rgb.shape[-1])
    l_eik = ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean()
    total = l_rgb * rgb_mse_weight + l_eik * eikonal_weight
    terms = {"rgb_mse": l_rgb, "eikonal": l_eik}
    if curvature_weight > 0:
        l_curv = out["sdf_laplace_samples"].abs().mean()
        total = total + l_curv * curvature_weight
        terms["curvature"] = l_curv
    return total, terms


class _NeusLoss(torch.autograd.Function):
    """loss_terms in two launches (angelo_neus_loss_fwd/bwd): returns (total,
    rgb_mse, eikonal, curvature); only the total carries a gradient."""

    _ws = {}

    @staticmethod
    def forward(ctx, rgb_pred, rgb_true, valid, sdf_grad, laplace, w_rgb, w_eik, w_curv):
        from . import _lib
        from .ops import _p, _s
        dev = rgb_pred.device
        ws = _NeusLoss._ws.get(dev)
        if ws is None:
            ws = torch.zeros(_lib.raw("angelo_loss_workspace_size")(), dtype=torch.uint8, device=dev)
            _NeusLoss._ws[dev] = ws
        c = rgb_pred.detach().float().contiguous()
        t = rgb_true.detach().float().contiguous()
        v = valid.reshape(-1).to(torch.bool).contiguous()
        g = sdf_grad.detach().float().contiguous()
        lap = laplace.detach().float().contiguous().reshape(-1) if laplace is not None else None
        out = torch.empty(5, device=dev)
        _lib.call("angelo_neus_loss_fwd", _p(c), _p(t), _p(v), c.shape[0], _p(g),
                  _p(lap) if lap is not None else None, g.shape[0], float(w_rgb), float(w_eik),
                  float(w_curv), _p(ws), _p(out), _s(dev))
        ctx.save_for_backward(c, t, v, g, lap if lap is not None else torch.empty(0, device=dev), out)
        ctx.has_lap = lap is not None
        ctx.w = (float(w_rgb), float(w_eik), float(w_curv))
        ctx.lap_shape = laplace.shape if laplace is not None else None
        terms = out[1:4].clone()
        ctx.mark_non_differentiable(terms)
        return out[0].clone(), terms

    @staticmethod
    def backward(ctx, d_total, d_terms):
        from . import _lib
        from .ops import _p, _s
        c, t, v, g, lap, stats = ctx.saved_tensors
        dev = c.device
        dt = (d_total if d_total is not None else torch.zeros((), device=dev)).float().reshape(1).contiguous()
        d_c = torch.empty_like(c)
        d_g = torch.empty_like(g)
        d_lap = torch.empty_like(lap) if ctx.has_lap else None
        _lib.call("angelo_neus_loss_bwd", _p(c), _p(t), _p(v), c.shape[0], _p(g),
                  _p(lap) if ctx.has_lap else None, g.shape[0], *ctx.w, _p(stats), _p(dt), _p(d_c),
                  _p(d_g), _p(d_lap) if d_lap is not None else None, _s(dev))
        return (d_c, None, None, d_g, d_lap.view(ctx.lap_shape) if d_lap is not None else None,
                None, None, None)


def fused_loss_terms(out, rgb, eikonal_weight=0.1, curvature_weight=5e-4, rgb_mse_weight=10.0):
    """loss_terms through the native loss (same terms and weights)."""
    lap = out["sdf_laplace_samples"] if curvature_weight > 0 else None
    total, t = _NeusLoss.apply(out["comp_rgb_full"], rgb, out["rays_valid_full"][..., 0],
                               out["sdf_grad_samples"], lap, rgb_mse_weight, eikonal_weight,
                               curvature_weight)
    terms = {"rgb_mse": t[0], "eikonal": t[1]}
    if curvature_weight > 0:
        terms["curvature"] = t[2]
    return total, terms


# lambda_* keys of the reference's loss config (systems/neus.py:130-196) that
# this step does not compute; each names the term it weights.  lambda_normal
# belongs to the sdf_l1 term (it is added inside that branch, :182-194).
UNSUPPORTED_LOSS_TERMS = {
    "lambda_rgb_l1": "rgb L1 (systems/neus.py:134-136)",
    "lambda_mask": "foreground-mask BCE (systems/neus.py:142-145)",
    "lambda_opaque": "opacity BCE (systems/neus.py:147-149)",
    "lambda_sparsity": "SDF sparsity (systems/neus.py:151-153)",
    "lambda_distortion": "distortion (systems/neus.py:163-166)",
    "lambda_distortion_bg": "background distortion (systems/neus.py:168-171)",
    "lambda_sdf_l1": "SDF L1 + normal on SfM points (systems/neus.py:180-194)",
}


def unsupported_loss_terms(loss_cfg, global_step, has_mask=True):
    """The loss terms a config asks for at global_step (scheduled weight > 0)
    that this step does not compute, as {key: description}.  The mask term
    counts only when the data has masks (the reference multiplies it by 0
    otherwise, systems/neus.py:145)."""
    out = {}
    for key, what in UNSUPPORTED_LOSS_TERMS.items():
        if key not in loss_cfg:
            continue
        if key == "lambda_mask" and not has_mask:
            continue
        if scheduled_value(loss_cfg[key], global_step) > 0:
            out[key] = what
    return out


class NeuSTrainer:
    """One training step = update_step (band mask, FD eps, cosine anneal,
    occupancy refresh every 16 steps) -> forward -> losses -> backward ->
    AdamW (angelo_gb.optim, one native pass per parameter).  Ray counts follow
    the reference's dynamic sampling rule.

    The step computes the rgb MSE, eikonal and curvature terms; a loss config
    that gives any other term a weight > 0 at the current step raises
    NotImplementedError instead of training a different objective
    (has_mask: whether the rays come with foreground masks, which the
    reference's mask term needs)."""

    def __init__(self, model, system_config=None, train_num_rays=256, max_train_num_rays=8192,
                 train_num_samples=1 << 18, dynamic_ray_sampling=True, has_mask=True):
        self.model = model
        sc = to_config(system_config or {})
        self.loss_cfg = to_config(sc.get("loss", {}))
        self.has_mask = bool(has_mask)
        self._check_loss(0)
        opt = to_config(sc.get("optimizer", {}))
        args = dict(opt.get("args", {"lr": 0.01, "betas": [0.9, 0.99], "eps": 1e-15}))
        groups = []
        per = opt.get("params", {"geometry": {"lr": 0.01}, "texture": {"lr": 0.01},
                                 "variance": {"lr": 0.001}})
        for name, a in per.items():
            mod = getattr(model, name, None)
            if mod is None:
                continue
            params = list(mod.parameters()) if isinstance(mod, torch.nn.Module) else [mod]
            groups.append({"params": params, "name": name, **a})
        args["betas"] = tuple(args.get("betas", (0.9, 0.99)))
        self.optimizer = AdamW(groups, **args)
        self.train_num_rays = int(train_num_rays)
        self.max_train_num_rays = int(max_train_num_rays)
        self.train_num_samples = int(train_num_samples)
        self.dynamic = dynamic_ray_sampling
        self.global_step = 0

    def C(self, v):
        return scheduled_value(v, self.global_step)

    def _check_loss(self, step):
        bad = unsupported_loss_terms(self.loss_cfg, step, self.has_mask)
        if bad:
            raise NotImplementedError(
                "loss terms with a non-zero weight at step %d are not computed by this training "
                "step: %s" % (step, "; ".join(f"{k} = {v}" for k, v in bad.items())))

    def step(self, rays, rgb, background_color):
        self._check_loss(self.global_step)
        m = self.model
        m.update_step(0, self.global_step)
        m.background_color = background_color
        out = m(rays)
        # the march sized its outputs on the host: no device read here, so
        # the backward is enqueued while the forward still runs
        n_samples = getattr(m, "last_num_samples", None)
        if n_samples is None:
            n_samples = int(out["num_samples_full"].sum().item())
        if self.dynamic:
            new = int(self.train_num_rays * (self.train_num_samples / max(n_samples, 1)))
            self.train_num_rays = min(int(self.train_num_rays * 0.9 + new * 0.1),
                                      self.max_train_num_rays)
        lc = self.loss_cfg
        fn = fused_loss_terms if getattr(m, "fused", False) else loss_terms
        loss, terms = fn(out, rgb,
                         eikonal_weight=self.C(lc.get("lambda_eikonal", 0.1)),
                         curvature_weight=self.C(lc.get("lambda_curvature", 5e-4)),
                         rgb_mse_weight=self.C(lc.get("lambda_rgb_mse", 10.0)))
        self.optimizer.zero_grad(set_to_none=True)
        loss.backward()
        self.optimizer.step()
        self.global_step += 1
        return loss.detach(), n_samples
