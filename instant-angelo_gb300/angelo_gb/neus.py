"""Drop-in for NeuSModel (models/neus.py:46-318), registered as 'neus', with
its VarianceNetwork (:15-43) and the nerfacc 0.3.3 OccupancyGrid it drives
(:63-68, 108-109).  Ray marching, occupancy update, transmittance weights and
accumulation run in libangelo_gb.so; with ``fused: true`` the per-sample
geometry, radiance and compositing run in the fused kernels
(angelo_gb.fused)."""
from __future__ import annotations

import math
from collections import defaultdict

import torch
import torch.nn as nn
import torch.nn.functional as F

from . import _lib, models, ops
from .config import to_config


class VarianceNetwork(nn.Module):
    """inv_s = exp(10 * variance), optionally clamped by the modulation
    schedule (models/neus.py:15-43)."""

    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        self.init_val = config.init_val
        self.register_parameter("variance", nn.Parameter(torch.tensor(float(config.init_val))))
        self.modulate = config.get("modulate", False)
        self.do_mod = False
        if self.modulate:
            self.mod_start_steps = config.mod_start_steps
            self.reach_max_steps = config.reach_max_steps
            self.max_inv_s = config.max_inv_s

    @property
    def inv_s(self):
        val = torch.exp(self.variance * 10.0)
        if self.modulate and self.do_mod:
            val = val.clamp_max(self.mod_val)
        return val

    def forward(self, x):
        return torch.ones([len(x), 1], device=self.variance.device) * self.inv_s

    def update_step(self, epoch, global_step):
        if self.modulate:
            self.do_mod = global_step > self.mod_start_steps
            if not self.do_mod:
                self.prev_inv_s = self.inv_s.item()
            else:
                self.mod_val = min((global_step / self.reach_max_steps) *
                                   (self.max_inv_s - self.prev_inv_s) + self.prev_inv_s,
                                   self.max_inv_s)


class OccupancyGrid(nn.Module):
    """res^3 occupancy grid over an AABB: float occupancies updated by EMA and a
    1-bit-per-cell mask read by the marcher (nerfacc 0.3.3 semantics: all cells
    during warm-up, then num_cells/4 uniform + as many occupied cells; the
    threshold is min(mean(occs), occ_thre))."""

    def __init__(self, roi_aabb, resolution=128, contraction_type="aabb"):
        super().__init__()
        self.res = int(resolution)
        self.num_cells = self.res ** 3
        self.register_buffer("roi_aabb", torch.as_tensor(roi_aabb, dtype=torch.float32).clone())
        # host copy of the box, so that a march needs no device read
        self.roi = tuple(float(v) for v in self.roi_aabb)
        self.register_buffer("occs", torch.zeros(self.num_cells))
        self.register_buffer("bits", torch.zeros((self.num_cells + 31) // 32, dtype=torch.int32))
        self.contraction_type = contraction_type
        self.jitter_fn = lambda t: torch.rand_like(t, dtype=torch.float32)

    def _load_from_state_dict(self, state_dict, prefix, *args, **kwargs):
        super()._load_from_state_dict(state_dict, prefix, *args, **kwargs)
        self.roi = tuple(float(v) for v in self.roi_aabb.cpu())

    @property
    def binary(self):
        b = self.bits.view(-1, 1).bitwise_right_shift(
            torch.arange(32, device=self.bits.device, dtype=torch.int32)) & 1
        return b.reshape(-1)[: self.num_cells].bool().view(self.res, self.res, self.res)

    def cell_coords(self, idx):
        r = self.res
        return torch.stack([idx // (r * r), (idx // r) % r, idx % r], -1)

    @torch.no_grad()
    def sample_cells(self, step, warmup_steps):
        dev = self.occs.device
        if step < warmup_steps:
            return torch.arange(self.num_cells, device=dev)
        n = self.num_cells // 4
        uni = torch.randint(self.num_cells, (n,), device=dev)
        occ_idx = torch.nonzero(self.binary.flatten())[:, 0]
        if n < len(occ_idx):
            occ_idx = occ_idx[torch.randint(len(occ_idx), (n,), device=dev)]
        return torch.cat([uni, occ_idx])

    @property
    def contraction(self):
        return (_lib.CONTRACT_UNBOUNDED_SPHERE if self.contraction_type == "unbounded_sphere"
                else _lib.CONTRACT_AABB)

    @torch.no_grad()
    def update(self, step, occ_eval_fn, occ_thre=0.01, ema_decay=0.95, warmup_steps=256):
        idx = self.sample_cells(step, warmup_steps)
        coords = self.cell_coords(idx).float()
        x = (coords + self.jitter_fn(coords)) / self.res
        lo, hi = self.roi_aabb[:3], self.roi_aabb[3:]
        if self.contraction_type == "unbounded_sphere":
            # only the cells inside the contracted ball are valid; [0,1]^3 ->
            # [-2,2]^3 -> inverse sphere contraction -> [-1,1]^3 -> roi
            keep = (x - 0.5).norm(dim=-1) < 0.5
            x, idx = x[keep], idx[keep]
            u = x * 4.0 - 2.0
            nrm = u.norm(dim=-1, keepdim=True)
            u = torch.where(nrm > 1.0, u / (nrm * (2.0 - nrm)), u)
            x = u * 0.5 + 0.5
        x = x * (hi - lo) + lo
        occ = occ_eval_fn(x).reshape(-1).float()
        ops.occ_update(self.occs, idx, occ, ema_decay, occ_thre, self.bits)

    @torch.no_grad()
    def every_n_step(self, step, occ_eval_fn, occ_thre=1e-2, ema_decay=0.95, warmup_steps=256,
                     n=16):
        if not self.training:
            raise RuntimeError("the occupancy grid is only updated in training mode")
        if step % n == 0:
            self.update(step, occ_eval_fn, occ_thre, ema_decay, warmup_steps)


def chunk_batch(func, chunk_size, move_to_cpu, *args, **kwargs):
    """models/utils.py:14-51: run func over chunks of the leading dim."""
    B = next(a.shape[0] for a in args if isinstance(a, torch.Tensor))
    out = defaultdict(list)
    out_type = None
    for i in range(0, B, chunk_size):
        oc = func(*[a[i:i + chunk_size] if isinstance(a, torch.Tensor) else a for a in args],
                  **kwargs)
        if oc is None:
            continue
        out_type = type(oc)
        if isinstance(oc, torch.Tensor):
            oc = {0: oc}
        elif isinstance(oc, (tuple, list)):
            n = len(oc)
            oc = dict(enumerate(oc))
        for k, v in oc.items():
            v = v if torch.is_grad_enabled() else v.detach()
            out[k].append(v.cpu() if move_to_cpu else v)
    if out_type is None:
        return None
    out = {k: torch.cat(v, dim=0) for k, v in out.items()}
    if out_type is torch.Tensor:
        return out[0]
    if out_type in (tuple, list):
        return out_type([out[i] for i in range(n)])
    return out


def fused_radiance_bg(texture):
    """Whether the learned background's texture runs on the fused radiance
    kernel: a VolumeRadiance (models/texture.py:10-30) on [feature,
    SH4((d+1)/2)] with a sigmoid colour and a ReLU VanillaMLP of two hidden
    layers of 64, whose input width the kernel is instantiated for."""
    net = getattr(texture, "network", None)
    cfg = texture.config
    if type(texture).__name__ != "VolumeRadiance" or net is None:
        return False
    feat = int(cfg.input_feature_dim)
    return (not net.sphere_init and not net.weight_norm and net.n_neurons == 64
            and net.n_hidden_layers == 2 and net.output_activation in (None, "none", "None")
            and str(cfg.get("color_activation", "")).lower() == "sigmoid"
            and texture.n_dir_dims == 3 and texture.encoding.n_output_dims == 16
            and net.dim_in == feat + 16 and (feat + 19 + 15) // 16 in (2, 3, 6))


@models.register("neus")
class NeuSModel(nn.Module):
    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        fused = bool(config.get("fused", False))
        config.geometry["fused"] = fused
        config.texture["fused"] = fused
        for k in ("fused_precision", "fused_table_dtype"):
            if k in config:
                config.geometry[k] = config[k]
        self.fused = fused
        self.geometry = models.make(config.geometry.name, config.geometry)
        self.texture = models.make(config.texture.name, config.texture)
        # forward MLP arithmetic of the fused kernels: "fp32" (default,
        # bf16x3), "fp16" (one fp16 pass: the precision form) or "bf16" (one
        # bf16 pass)
        self.texture.fused_precision = config.get("fused_precision", "fp32")
        self.geometry.contraction_type = "aabb"
        self.learned_background = bool(config.get("learned_background", False))
        if self.learned_background:
            # models/neus.py:51-56: density field and radiance outside the box,
            # marched from the box exit (or 0.1) to 1e3 with exponential steps
            config.geometry_bg["fused"] = fused
            self.geometry_bg = models.make(config.geometry_bg.name, config.geometry_bg)
            self.texture_bg = models.make(config.texture_bg.name, config.texture_bg)
            self.geometry_bg.contraction_type = "unbounded_sphere"
            self.near_plane_bg, self.far_plane_bg = 0.1, 1e3
            self.cone_angle_bg = 10 ** (math.log10(self.far_plane_bg) / config.num_samples_per_ray_bg) - 1.0
            self.render_step_size_bg = 0.01
        self.variance = VarianceNetwork(config.variance)
        r = config.radius
        self.register_buffer("scene_aabb", torch.as_tensor([-r, -r, -r, r, r, r],
                                                           dtype=torch.float32))
        if config.grid_prune:
            self.occupancy_grid = OccupancyGrid(self.scene_aabb, resolution=128)
            if self.learned_background:
                self.occupancy_grid_bg = OccupancyGrid(self.scene_aabb, resolution=256,
                                                       contraction_type="unbounded_sphere")
        self.randomized = config.randomized
        self.background_color = None
        self.render_step_size = config.get("render_step_size",
                                           1.732 * 2 * config.radius / config.num_samples_per_ray)
        # near/far planes: absent in the reference's NeuS call (models/neus.py:215);
        # optional here for scenes marched between fixed planes without a grid
        self.near_plane = config.get("near_plane", None)
        self.far_plane = config.get("far_plane", None)
        self.cos_anneal_ratio = 1.0
        self.max_march_steps = int(config.get("max_march_steps", 1 << 20))
        self.stratified_fn = torch.rand_like

    # ------------------------------------------------------------- schedule
    def update_step(self, epoch, global_step):
        self.geometry.update_step(epoch, global_step)
        self.texture.update_step(epoch, global_step)
        if self.learned_background:
            self.geometry_bg.update_step(epoch, global_step)
            self.texture_bg.update_step(epoch, global_step)
        self.variance.update_step(epoch, global_step)
        cae = self.config.get("cos_anneal_end", 0)
        self.cos_anneal_ratio = 1.0 if cae == 0 else min(1.0, global_step / cae)

        def occ_eval_fn(x):
            sdf = self.geometry(x, with_grad=False, with_feature=False)
            inv_s = self.variance(torch.zeros([1, 3]))[:, :1].clip(1e-6, 1e6)
            inv_s = inv_s.expand(sdf.shape[0], 1)
            nxt = sdf[..., None] - self.render_step_size * 0.5
            prv = sdf[..., None] + self.render_step_size * 0.5
            pc = torch.sigmoid(prv * inv_s)
            nc = torch.sigmoid(nxt * inv_s)
            return ((pc - nc + 1e-5) / (pc + 1e-5)).view(-1, 1).clip(0.0, 1.0)

        def occ_eval_fn_bg(x):
            # density * step: the first-order 1 - exp(-density * step) (models/neus.py:103-106)
            density, _ = self.geometry_bg(x)
            return density[..., None] * self.render_step_size_bg

        if self.training and self.config.grid_prune:
            self.occupancy_grid.every_n_step(step=global_step, occ_eval_fn=occ_eval_fn,
                                             occ_thre=self.config.get("grid_prune_occ_thre", 0.01))
            if self.learned_background:
                self.occupancy_grid_bg.every_n_step(
                    step=global_step, occ_eval_fn=occ_eval_fn_bg,
                    occ_thre=self.config.get("grid_prune_occ_thre_bg", 0.01))

    def isosurface(self):
        return self.geometry.isosurface()

    # ---------------------------------------------------------------- render
    def get_alpha(self, sdf, normal, dirs, dists):
        """models/neus.py:117-139."""
        inv_s = self.variance(torch.zeros([1, 3]))[:, :1].clip(1e-6, 1e6)
        inv_s = inv_s.expand(sdf.shape[0], 1)
        true_cos = (dirs * normal).sum(-1, keepdim=True)
        r = self.cos_anneal_ratio
        iter_cos = -(F.relu(-true_cos * 0.5 + 0.5) * (1.0 - r) + F.relu(-true_cos) * r)
        nxt = sdf[..., None] + iter_cos * dists.reshape(-1, 1) * 0.5
        prv = sdf[..., None] - iter_cos * dists.reshape(-1, 1) * 0.5
        pc = torch.sigmoid(prv * inv_s)
        nc = torch.sigmoid(nxt * inv_s)
        return ((pc - nc + 1e-5) / (pc + 1e-5)).view(-1).clip(0.0, 1.0)

    def _samples_bound(self):
        """Samples any ray can have: its clipped length over the step, + 2
        (the stratified start shifts near by up to one step)."""
        if self.near_plane is None and self.far_plane is None:
            length = 2.0 * math.sqrt(3.0) * float(self.config.radius)   # the box diagonal
        elif self.near_plane is not None and self.far_plane is not None:
            length = float(self.far_plane) - float(self.near_plane)
        else:
            return None
        return int(math.ceil(length / self.render_step_size)) + 2

    def march_rays(self, rays_o, rays_d):
        """nerfacc.ray_marching as called at models/neus.py:210-220."""
        prev_grad = torch.is_grad_enabled()
        with torch.no_grad():
            if self.near_plane is None and self.far_plane is None:
                t_min, t_max = ops.ray_aabb_intersect(rays_o, rays_d, self.scene_aabb)
            else:
                t_min = torch.zeros_like(rays_o[:, 0])
                t_max = torch.full_like(rays_o[:, 0], 1e10)
                if self.near_plane is not None:
                    t_min = t_min.clamp(min=self.near_plane)
                if self.far_plane is not None:
                    t_max = t_max.clamp(max=self.far_plane)
            if self.randomized:
                t_min = t_min + self.stratified_fn(t_min) * self.render_step_size
            if self.config.grid_prune:
                g = self.occupancy_grid
                grid = dict(roi=g.roi, res=(g.res,) * 3, bits=g.bits)
            else:
                grid = dict(roi=ops.UNBOUNDED_ROI, res=(1, 1, 1), bits=None)
            before_read = None
            if self.fused and self.training:
                # the training step's weight preparation is enqueued while
                # the march's sample count travels to the host, so the GPU
                # runs it while the host sizes the outputs
                grad_mode = prev_grad

                def before_read():
                    from . import fused
                    with torch.set_grad_enabled(grad_mode):
                        fused.prepare_ahead(self)
            ri, t0, t1, offsets, _ = ops.march(rays_o, rays_d, t_min, t_max, self.render_step_size,
                                               cone_angle=0.0, max_steps=self.max_march_steps,
                                               max_samples_per_ray=self._samples_bound(),
                                               before_read=before_read, **grid)
        self._last_march = (t_min, t_max)
        self._n_fg = int(t0.shape[0])   # host-side, no device read
        return ri, t0, t1, offsets

    @property
    def last_num_samples(self):
        """Samples of the last forward as the reference counts them for its
        dynamic ray count (num_samples_full, models/neus.py:275): the
        foreground's plus the learned background's kept samples, known on
        the host (None before the first forward)."""
        n = self.__dict__.get("_n_fg")
        return None if n is None else n + self.__dict__.get("_n_bg", 0)

    def forward_(self, rays):
        n_rays = rays.shape[0]
        rays_o, rays_d = rays[:, 0:3].contiguous(), rays[:, 3:6].contiguous()
        bg_samples = None
        self._n_bg = 0
        if self.fused and self.learned_background:
            # the background's kept samples first: its two host reads (its
            # march's count, the kept count) then come before the foreground's
            # march, and the GPU runs the foreground's VolumeSDF forward while
            # the host enqueues the background's render and the loss
            bg_samples = self._bg_samples(rays_o, rays_d)
        ri, t0, t1, offsets = self.march_rays(rays_o, rays_d)
        if self.fused:
            from . import fused
            return fused.neus_forward(self, rays_o, rays_d, ri, t0, t1, offsets, n_rays,
                                      bg_samples=bg_samples)
        ray_indices = ri.long()
        t_origins = rays_o[ray_indices]
        t_dirs = rays_d[ray_indices]
        t_starts, t_ends = t0[:, None], t1[:, None]
        midpoints = (t_starts + t_ends) / 2.0
        positions = t_origins + t_dirs * midpoints
        dists = t_ends - t_starts
        sdf, sdf_grad, feature, sdf_laplace = self.geometry(positions, with_grad=True,
                                                            with_feature=True, with_laplace=True)
        normal = F.normalize(sdf_grad, p=2, dim=-1)
        alpha = self.get_alpha(sdf, normal, t_dirs, dists)[..., None]
        rgb = self.texture(feature, t_dirs, normal)
        weights = ops.render_weight_from_alpha(alpha, offsets)[:, None]
        opacity = ops.accumulate_along_rays(weights, offsets)
        depth = ops.accumulate_along_rays(weights, offsets, midpoints)
        comp_rgb = ops.accumulate_along_rays(weights, offsets, rgb)
        rays_fg = opacity > 0.1
        comp_normal = F.normalize(ops.accumulate_along_rays(weights, offsets, normal), p=2, dim=-1)
        comp_normal = torch.where(rays_fg, comp_normal, torch.zeros_like(comp_normal))
        out = {
            "comp_rgb": comp_rgb, "comp_normal": comp_normal, "opacity": opacity,
            "depth": depth, "rays_valid": opacity > 0,
            "num_samples": torch.full((1,), len(t0), dtype=torch.int32, device=rays.device),
        }
        if self.training:
            out.update({"sdf_samples": sdf, "sdf_grad_samples": sdf_grad,
                        "weights": weights.view(-1), "points": midpoints.view(-1),
                        "intervals": dists.view(-1), "ray_indices": ray_indices.view(-1),
                        "sdf_laplace_samples": sdf_laplace})
        return self._with_background(out, comp_rgb, rays_o, rays_d)

    def _bg_samples_bound(self):
        """Samples a background ray can have: the steps of the march
        recurrence from t = 0 to the far plane, + 4."""
        key = (self.render_step_size_bg, self.cone_angle_bg, self.far_plane_bg)
        if getattr(self, "_bg_bound", (None, 0))[0] == key:
            return self._bg_bound[1]
        t0, n = 0.0, 0
        step, cone = self.render_step_size_bg, self.cone_angle_bg
        t1 = t0 + max(t0 * cone, step)
        while (t0 + t1) * 0.5 < self.far_plane_bg:
            t0, t1 = t1, t1 + max(t1 * cone, step)
            n += 1
        self._bg_bound = (key, n + 4)
        return n + 4

    def _bg_samples(self, rays_o, rays_d):
        """The learned background's kept samples (no autograd graph): marched
        from the box exit (0.1 when the ray misses the box) to 1e3 through
        the unbounded-sphere grid, samples of transmittance < 1e-4 dropped
        (nerfacc's sigma_fn visibility test).  Returns (ray indices, t0, t1,
        offsets, reuse, and for the fused form's reuse the contracted points,
        the visibility pass's encodings and outputs and the kept rows)."""
        n_rays = rays_o.shape[0]
        pts_c = X_all = out_all = kidx = None
        with torch.no_grad():
            _, t_exit = ops.ray_aabb_intersect(rays_o, rays_d, self.scene_aabb)
            near = torch.where(t_exit > 1e9, torch.full_like(t_exit, self.near_plane_bg), t_exit)
            # nerfacc.ray_marching without scene_aabb: t in [0, 1e10], clamped by the planes
            t_min = torch.maximum(torch.zeros_like(near), near)
            t_max = torch.full_like(near, 1e10).clamp(max=self.far_plane_bg)
            if self.randomized:
                t_min = t_min + self.stratified_fn(t_min) * self.render_step_size_bg
            if self.config.grid_prune:
                g = self.occupancy_grid_bg
                grid = dict(roi=g.roi, res=(g.res,) * 3, bits=g.bits, contraction=g.contraction)
            else:
                grid = dict(roi=ops.UNBOUNDED_ROI, res=(1, 1, 1), bits=None)
            ri, t0, t1, offsets, _ = ops.march(rays_o, rays_d, t_min, t_max, self.render_step_size_bg,
                                               cone_angle=self.cone_angle_bg,
                                               max_steps=self.max_march_steps,
                                               max_samples_per_ray=self._bg_samples_bound(), **grid)
            reuse = self.fused and self.geometry_bg.fused_reuse_ok()
            native = reuse and self.geometry_bg.native_visibility_ok()
        if native:
            # the fused form: points, visibility test and compaction in native
            # launches (one device read, the kept count)
            from . import fused
            with torch.no_grad():
                pts_c = fused.bg_points(rays_o, rays_d, ri, t0, t1, self.geometry_bg.radius)
                X_all, out_all = self.geometry_bg.evaluate_contracted(pts_c)
                self._last_march_bg_full = (offsets, ri, t0, t1)
                ri, t0, t1, pts_c, out_all, kidx, offsets = fused.bg_visible(
                    out_all, float(self.geometry_bg.config.density_bias), ri, t0, t1, offsets, pts_c)
                self._last_march_bg = (offsets, ri, t0, t1)
        else:
            with torch.no_grad():
                rl = ri.long()
                pos = rays_o[rl] + rays_d[rl] * ((t0 + t1) * 0.5)[:, None]
                if reuse:
                    # the fused form keeps the visibility pass's encodings and
                    # outputs for the kept samples instead of evaluating them again
                    pts_c, X_all, out_all = self.geometry_bg.encode_and_evaluate(pos)
                    sigma, _ = self.geometry_bg.outputs(out_all)
                else:
                    sigma, _ = self.geometry_bg(pos)
                alpha = 1.0 - torch.exp(-sigma * (t1 - t0))
                keep = ops.transmittance_from_alpha(alpha, offsets) >= 1e-4
                self._last_march_bg_full = (offsets, ri, t0, t1)
                # the kept samples' indices once (one device read of their
                # count), then one gather per tensor
                kidx = keep.nonzero().squeeze(1)
                ri, t0, t1 = ri.index_select(0, kidx), t0.index_select(0, kidx), t1.index_select(0, kidx)
                if reuse:
                    # the encodings stay where they are: the backward reads the
                    # kept rows through kidx
                    pts_c, out_all = pts_c.index_select(0, kidx), out_all.index_select(0, kidx)
                offsets = ops.offsets_from_ray_indices(ri, n_rays)
                self._last_march_bg = (offsets, ri, t0, t1)
        self._n_bg = int(t0.shape[0])
        return ri, t0, t1, offsets, reuse, pts_c, X_all, out_all, kidx

    def forward_bg_(self, rays_o, rays_d, samples=None):
        """The learned background (models/neus.py:141-203): its kept samples
        (``_bg_samples``, or the ones given), then density, colour and weights
        from density."""
        n_rays = rays_o.shape[0]
        if samples is None:
            samples = self._bg_samples(rays_o, rays_d)
        ri, t0, t1, offsets, reuse, pts_c, X_all, out_all, kidx = samples
        ray_indices = ri.long()
        midpoints = ((t0 + t1) * 0.5)[:, None]
        intervals = (t1 - t0)[:, None]
        t_dirs = None
        if reuse:
            from . import fused
            density, feature = fused.density_field_reused(self.geometry_bg, pts_c, X_all, kidx, out_all)
        else:
            t_dirs = rays_d[ray_indices]
            positions = rays_o[ray_indices] + t_dirs * midpoints
            density, feature = self.geometry_bg(positions)
        if self.fused and fused_radiance_bg(self.texture_bg):
            # the radiance kernel takes the direction by ray index, as the
            # foreground's does
            from . import fused
            rgb = fused.radiance_forward(self.texture_bg, feature.contiguous(), None, ri,
                                         rays_d.contiguous())
        else:
            if t_dirs is None:
                t_dirs = rays_d[ray_indices]
            rgb = self.texture_bg(feature, t_dirs)
        if self.fused:
            from . import fused
            comp_rgb, opacity, depth, weights = fused.density_composite(
                density, rgb, t0, t1, offsets, self.background_color)
            weights = weights[:, None]
        else:
            weights = ops.render_weight_from_density(t0[:, None], t1[:, None], density[:, None], offsets)
            opacity = ops.accumulate_along_rays(weights, offsets)
            depth = ops.accumulate_along_rays(weights, offsets, midpoints)
            comp_rgb = ops.accumulate_along_rays(weights, offsets, rgb)
            comp_rgb = comp_rgb + self.background_color * (1.0 - opacity)
        out = {"comp_rgb": comp_rgb, "opacity": opacity, "depth": depth, "rays_valid": opacity > 0,
               "num_samples": torch.full((1,), len(t0), dtype=torch.int32, device=rays_o.device)}
        if self.training:
            out.update({"weights": weights.view(-1), "points": midpoints.view(-1),
                        "intervals": intervals.view(-1), "ray_indices": ray_indices.view(-1)})
        return out

    def background(self, out, comp_rgb, rays_o, rays_d, samples=None):
        """The background outputs: the learned background (on its kept
        samples when given), or the constant colour (models/neus.py:265-272)."""
        if self.learned_background:
            return self.forward_bg_(rays_o, rays_d, samples)
        bg = self.background_color
        return {"comp_rgb": bg[None, :].expand(*comp_rgb.shape),
                "num_samples": torch.zeros_like(out["num_samples"]),
                "rays_valid": torch.zeros_like(out["rays_valid"])}

    def _with_background(self, out, comp_rgb, rays_o=None, rays_d=None, bg_samples=None):
        bg = self.background_color
        if bg is None:
            raise RuntimeError("set model.background_color before rendering "
                               "(the reference's system sets it per batch)")
        out_bg = self.background(out, comp_rgb, rays_o, rays_d, bg_samples)
        out_full = {"comp_rgb": out["comp_rgb"] + out_bg["comp_rgb"] * (1.0 - out["opacity"]),
                    "num_samples": out["num_samples"] + out_bg["num_samples"],
                    "rays_valid": out["rays_valid"] | out_bg["rays_valid"]}
        return {**out, **{k + "_bg": v for k, v in out_bg.items()},
                **{k + "_full": v for k, v in out_full.items()}}

    def forward(self, rays):
        if self.training:
            out = self.forward_(rays)
        else:
            out = chunk_batch(self.forward_, self.config.ray_chunk, True, rays)
        return {**out, "inv_s": self.variance.inv_s}

    def train(self, mode=True):
        self.randomized = mode and self.config.randomized
        return super().train(mode=mode)

    def eval(self):
        self.randomized = False
        return super().eval()

    def regularizations(self, out):
        return {}

    @torch.no_grad()
    def export(self, export_config):
        """models/neus.py:309-318."""
        mesh = self.isosurface()
        if export_config.get("export_vertex_color", False):
            _, sdf_grad, features = chunk_batch(self.geometry, export_config.chunk_size, False,
                                                mesh["v_pos"].to(self.scene_aabb.device),
                                                with_grad=True, with_feature=True)
            mesh["v_rgb"] = torch.sigmoid(features[..., 1:4]).cpu()
            mesh["v_norm"] = F.normalize(sdf_grad, p=2, dim=-1).cpu()
        return mesh
