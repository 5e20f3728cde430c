"""Import the reference's own model code on the CPU with stand-ins for the
packages it needs but that are absent here (tinycudann, nerfacc 0.3.3,
pytorch_lightning, omegaconf, trimesh).

TEST INFRASTRUCTURE ONLY: used by ``tests/golden/make_golden.py`` to run the
reference's VolumeSDF / texture / NeuSModel code (models/geometry.py,
models/texture.py, models/neus.py, models/network_utils.py) exactly as written,
so that golden vectors pin this repository's oracle.  The tcnn and nerfacc
stand-ins are the oracle's restatements (``oracle/cref.py``,
``oracle/neus_fp64.py``); the reference-owned Python runs unmodified.

The reference tree is read-only: bytecode writing is disabled before import.
"""
from __future__ import annotations

import contextlib
import enum
import sys
import types

import numpy as np
import torch
import torch.nn as nn

from . import cref
from . import neus_fp64 as O

sys.dont_write_bytecode = True


class AttrDict(dict):
    """Minimal stand-in for an OmegaConf DictConfig: attribute access, .get()."""

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = v

    @staticmethod
    def wrap(d):
        if isinstance(d, dict):
            return AttrDict({k: AttrDict.wrap(v) for k, v in d.items()})
        if isinstance(d, list):
            return [AttrDict.wrap(v) for v in d]
        return d


def _to_container(c, resolve=True):
    if isinstance(c, dict):
        return {k: _to_container(v) for k, v in c.items()}
    if isinstance(c, list):
        return [_to_container(v) for v in c]
    return c


# --------------------------------------------------------------- tcnn stand-in


class _HashGridEncoding(nn.Module):
    """tcnn.Encoding(otype=HashGrid): flat ``params`` U(-1e-4, 1e-4) like tcnn."""

    def __init__(self, n_in, cfg):
        super().__init__()
        assert n_in == 3
        self.lay = O.HashGridLayout(cfg["n_levels"], cfg["n_features_per_level"],
                                    cfg["log2_hashmap_size"], cfg["base_resolution"],
                                    cfg["per_level_scale"])
        self.n_input_dims = n_in
        self.n_output_dims = self.lay.L * self.lay.F
        self.params = nn.Parameter(torch.empty(self.lay.n_params).uniform_(-1e-4, 1e-4))

    def forward(self, x):
        out = O.hash_encode(x.double(), self.params.double(), self.lay)
        return out.float()


class _SHEncoding(nn.Module):
    def __init__(self, n_in, cfg):
        super().__init__()
        assert cfg["degree"] == 4
        self.n_input_dims = n_in
        self.n_output_dims = 16

    def forward(self, x):
        return O.sh4(x.double()).float()


def _tcnn_encoding(n_in, cfg):
    if cfg["otype"] == "HashGrid":
        return _HashGridEncoding(n_in, cfg)
    if cfg["otype"] == "SphericalHarmonics":
        return _SHEncoding(n_in, cfg)
    raise NotImplementedError(cfg["otype"])


# ------------------------------------------------------------ nerfacc stand-in


class ContractionType(enum.Enum):
    AABB = 0
    UN_BOUNDED_TANH = 1
    UN_BOUNDED_SPHERE = 2


class OccupancyGrid(nn.Module):
    """nerfacc 0.3.3 OccupancyGrid (models/neus.py:63-68,108-109)."""

    def __init__(self, roi_aabb, resolution=128, contraction_type=ContractionType.AABB):
        super().__init__()
        self.res = int(resolution)
        self.num_cells = self.res ** 3
        self.register_buffer("roi_aabb", torch.as_tensor(roi_aabb, dtype=torch.float32))
        self.register_buffer("occs", torch.zeros(self.num_cells))
        self.register_buffer("binary", torch.zeros(self.res, self.res, self.res, dtype=torch.bool))
        g = torch.arange(self.res)
        gx, gy, gz = torch.meshgrid(g, g, g, indexing="ij")
        self.grid_coords = torch.stack([gx, gy, gz], -1).reshape(-1, 3)
        self.contraction_type = contraction_type
        self.record = None

    @torch.no_grad()
    def every_n_step(self, step, occ_eval_fn, occ_thre=1e-2, ema_decay=0.95, warmup_steps=256,
                     n=16):
        if step % n != 0:
            return
        if step < warmup_steps:
            idx = torch.arange(self.num_cells)
        else:
            N = self.num_cells // 4
            uni = torch.randint(self.num_cells, (N,))
            occ_idx = torch.nonzero(self.binary.flatten())[:, 0]
            if N < len(occ_idx):
                occ_idx = occ_idx[torch.randint(len(occ_idx), (N,))]
            idx = torch.cat([uni, occ_idx])
        gc = self.grid_coords[idx]
        jit = torch.rand_like(gc, dtype=torch.float32)
        x = (gc + jit) / self.res
        lo, hi = self.roi_aabb[:3], self.roi_aabb[3:]
        x = x * (hi - lo) + lo
        occ = occ_eval_fn(x).squeeze(-1)
        self.record = {"indices": idx.numpy().copy(), "jitter": jit.numpy().copy(),
                       "occ_eval": occ.numpy().copy()}
        self.occs[idx] = torch.maximum(self.occs[idx] * ema_decay, occ)
        self.binary = (self.occs > torch.clamp(self.occs.mean(), max=occ_thre)).view(self.binary.shape)


_MARCH_RECORD = {}


def ray_aabb_intersect(rays_o, rays_d, aabb):
    a, b = cref.ray_aabb(rays_o.numpy(), rays_d.numpy(), aabb.numpy())
    return torch.from_numpy(a), torch.from_numpy(b)


def ray_marching(rays_o, rays_d, t_min=None, t_max=None, scene_aabb=None, grid=None,
                 sigma_fn=None, alpha_fn=None, early_stop_eps=1e-4, alpha_thre=0.0,
                 near_plane=None, far_plane=None, render_step_size=1e-3, stratified=False,
                 cone_angle=0.0):
    assert sigma_fn is None and alpha_fn is None
    if t_min is None or t_max is None:
        if scene_aabb is not None:
            t_min, t_max = ray_aabb_intersect(rays_o, rays_d, scene_aabb)
        else:
            t_min = torch.zeros_like(rays_o[..., 0])
            t_max = torch.ones_like(rays_o[..., 0]) * 1e10
    if near_plane is not None:
        t_min = torch.clamp(t_min, min=near_plane)
    if far_plane is not None:
        t_max = torch.clamp(t_max, max=far_plane)
    if stratified:
        jit = torch.rand_like(t_min)
        _MARCH_RECORD["jitter"] = jit.numpy().copy()
        t_min = t_min + jit * render_step_size
    if grid is not None:
        roi = grid.roi_aabb.numpy()
        binary = grid.binary.numpy().astype(np.uint8)
    else:
        roi = np.array([-1e10, -1e10, -1e10, 1e10, 1e10, 1e10], np.float32)
        binary = np.ones((1, 1, 1), np.uint8)
    _MARCH_RECORD["t_min"] = t_min.numpy().copy()
    _MARCH_RECORD["t_max"] = t_max.numpy().copy()
    counts, offsets, ri, t0, t1, _ = cref.march(rays_o.detach().numpy(), rays_d.detach().numpy(),
                                                t_min.numpy(), t_max.numpy(), roi, binary,
                                                render_step_size, cone_angle)
    _MARCH_RECORD["offsets"] = offsets
    return (torch.from_numpy(ri.astype(np.int32)), torch.from_numpy(t0)[:, None],
            torch.from_numpy(t1)[:, None])


def _offsets_from_indices(ray_indices, n_rays):
    cnt = torch.bincount(ray_indices.long(), minlength=n_rays)
    off = torch.zeros(n_rays + 1, dtype=torch.int64)
    off[1:] = torch.cumsum(cnt, 0)
    return off


def render_weight_from_alpha(alphas, packed_info=None, ray_indices=None, n_rays=None,
                             early_stop_eps=1e-4, alpha_thre=0.0):
    a = alphas.reshape(-1)
    off = _offsets_from_indices(ray_indices, n_rays).tolist()
    parts = []
    for r in range(n_rays):
        seg = a[off[r]:off[r + 1]]
        if seg.numel() == 0:
            continue
        T = torch.cumprod(torch.cat([torch.ones(1, dtype=seg.dtype), 1 - seg[:-1]]), 0)
        parts.append(seg * T * (T >= early_stop_eps).to(seg.dtype))
    w = torch.cat(parts) if parts else a * 0
    return w.reshape(alphas.shape)


def render_weight_from_density(*a, **k):
    raise NotImplementedError("learned background is outside the hot path")


def accumulate_along_rays(weights, ray_indices, values=None, n_rays=None):
    src = weights if values is None else weights * values
    out = torch.zeros((n_rays, src.shape[-1]), dtype=src.dtype)
    return out.index_add(0, ray_indices.long(), src)


# ---------------------------------------------------------------- installation


def install(reference_root, kernel_modules=None):
    """Insert the stand-in modules and import the reference's ``models``
    package from ``reference_root``.  Returns the imported ``models`` module.
    kernel_modules ({name: module} for tinycudann, nerfacc and
    nerfacc.intersection, e.g. angelo_gb.seam.modules()) replaces the
    oracle's tcnn / nerfacc restatements."""
    def mod(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    if kernel_modules is not None:
        sys.modules.update(kernel_modules)
    else:
        mod("tinycudann", Encoding=_tcnn_encoding, Network=None,
            NetworkWithInputEncoding=None, free_temporary_memory=lambda: None)
        nerfacc = mod("nerfacc", ContractionType=ContractionType, OccupancyGrid=OccupancyGrid,
                      ray_marching=ray_marching, render_weight_from_alpha=render_weight_from_alpha,
                      render_weight_from_density=render_weight_from_density,
                      accumulate_along_rays=accumulate_along_rays)
        nerfacc.intersection = mod("nerfacc.intersection", ray_aabb_intersect=ray_aabb_intersect)
    noop = lambda *a, **k: None  # noqa: E731
    pl = mod("pytorch_lightning", LightningModule=nn.Module)
    pl.utilities = mod("pytorch_lightning.utilities")
    pl.utilities.rank_zero = mod("pytorch_lightning.utilities.rank_zero", rank_zero_info=noop,
                                 rank_zero_debug=noop, rank_zero_only=lambda f: f)
    oc = mod("omegaconf")
    oc.OmegaConf = types.SimpleNamespace(register_new_resolver=noop, to_container=_to_container)
    mod("trimesh")
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    for pkg in ("systems", "utils"):
        m = types.ModuleType(pkg)
        m.__path__ = [f"{reference_root}/{pkg}"]
        sys.modules[pkg] = m
    import utils.misc as misc  # noqa: E402
    misc.get_rank = lambda: "cpu"
    torch.cuda.device = lambda *_a, **_k: contextlib.nullcontext()
    import models  # noqa: E402
    return models
