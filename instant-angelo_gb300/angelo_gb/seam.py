"""The library seam: stand-ins for the two CUDA packages the reference reaches
its hot path through -- tiny-cuda-nn (``import tinycudann as tcnn``,
models/network_utils.py:6, models/utils.py:11) and nerfacc 0.3.3 (``from
nerfacc import ...``, models/neus.py:11-12, models/geometry.py:15) -- with
their names and call signatures, backed by libangelo_gb.so.

``install()`` registers them in ``sys.modules`` as ``tinycudann``,
``nerfacc`` and ``nerfacc.intersection``, so that the reference's own model
code (models/network_utils.py, models/geometry.py, models/texture.py,
models/neus.py), imported afterwards and unmodified, runs on this library's
kernels:

* ``tinycudann.Encoding(n_input_dims, config)``: HashGrid (flat ``params``
  initialised U(-1e-4, 1e-4), encode forward and table scatter-add backward
  on angelo_hashgrid_fwd/bwd) and SphericalHarmonics degree 4
  (angelo_sh4_fwd/bwd).  Outputs are float32 (tcnn's half-precision build
  returns float16, which the reference promotes to float32 at its next
  operation).
* ``nerfacc``: ``ContractionType``, ``OccupancyGrid`` (EMA update and bit
  packing on angelo_occ_update), ``ray_marching`` (angelo_march_*: AABB clip,
  near / far planes, stratified jitter, occupancy skipping, cone angle, the
  unbounded-sphere contraction, and the sigma_fn / alpha_fn visibility test
  on angelo_weights_fwd's transmittance), ``render_weight_from_alpha``,
  ``render_weight_from_density``, ``accumulate_along_rays`` (with their
  backward kernels) and ``intersection.ray_aabb_intersect``.

Entry points of tcnn that no shipped configuration reaches (``Network``,
``NetworkWithInputEncoding``, other encodings) raise NotImplementedError
when called; nothing falls back to another implementation."""
from __future__ import annotations

import enum
import sys
import types

import torch
import torch.nn as nn

from . import network_utils, ops
from .neus import OccupancyGrid as _OccupancyGrid

# ------------------------------------------------------------------ tinycudann


class _HashGrid(network_utils.HashGridEncoding):
    """tcnn.Encoding(otype=HashGrid): x (N, 3) in [0, 1] -> (N, L*F), every
    level active (the reference applies its band mask afterwards,
    models/network_utils.py:56-59); the table is ``params`` as in tcnn."""

    def forward(self, x):
        return super().forward(x.reshape(-1, 3))


def Encoding(n_input_dims, encoding_config, seed=1337, dtype=None):  # noqa: N802
    """tcnn.Encoding: the HashGrid and degree-4 SphericalHarmonics encodings
    the reference's configurations use (models/network_utils.py:47,91)."""
    otype = encoding_config["otype"]
    if otype in ("HashGrid", "Grid") and encoding_config.get("type", "Hash") == "Hash":
        return _HashGrid(n_input_dims, encoding_config)
    if otype == "SphericalHarmonics":
        return network_utils.SphericalHarmonicsEncoding(n_input_dims, encoding_config)
    raise NotImplementedError(f"tinycudann.Encoding otype {otype!r} is not provided by libangelo_gb")


def Network(*args, **kwargs):  # noqa: N802
    raise NotImplementedError("tinycudann.Network (fully fused MLP): the reference's configurations "
                              "use VanillaMLP; libangelo_gb provides no tcnn network")


def NetworkWithInputEncoding(*args, **kwargs):  # noqa: N802
    raise NotImplementedError("tinycudann.NetworkWithInputEncoding is not provided by libangelo_gb")


def free_temporary_memory():
    """tcnn frees its scratch arenas here (models/utils.py:120); this library
    keeps none."""


# --------------------------------------------------------------------- nerfacc


class ContractionType(enum.Enum):
    """nerfacc 0.3.3 ContractionType."""
    AABB = 0
    UN_BOUNDED_TANH = 1
    UN_BOUNDED_SPHERE = 2


class OccupancyGrid(_OccupancyGrid):
    """nerfacc.OccupancyGrid(roi_aabb, resolution, contraction_type)
    (models/neus.py:63-74)."""

    def __init__(self, roi_aabb, resolution=128, contraction_type=ContractionType.AABB):
        if isinstance(resolution, (list, tuple)):
            if len(set(resolution)) != 1:
                raise NotImplementedError("the occupancy grid is cubic")
            resolution = resolution[0]
        if contraction_type == ContractionType.UN_BOUNDED_TANH:
            raise NotImplementedError("the UN_BOUNDED_TANH contraction is not on the hot path")
        name = "unbounded_sphere" if contraction_type == ContractionType.UN_BOUNDED_SPHERE else "aabb"
        super().__init__(torch.as_tensor(roi_aabb, dtype=torch.float32).reshape(6).cpu(),
                         int(resolution), name)


def ray_aabb_intersect(rays_o, rays_d, aabb):
    """nerfacc.intersection.ray_aabb_intersect (models/neus.py:12,153)."""
    return ops.ray_aabb_intersect(rays_o.contiguous(), rays_d.contiguous(), aabb)


def _offsets(ray_indices, n_rays):
    return ops.offsets_from_ray_indices(ray_indices, n_rays)


def _n_rays(ray_indices, n_rays):
    if n_rays is not None:
        return int(n_rays)
    return int(ray_indices.max().item()) + 1 if ray_indices.numel() else 0


@torch.no_grad()
def ray_marching(rays_o, rays_d, t_min=None, t_max=None, scene_aabb=None, grid=None, sigma_fn=None,
                 alpha_fn=None, early_stop_eps=1e-4, alpha_thre=0.0, near_plane=None,
                 far_plane=None, render_step_size=1e-3, stratified=False, cone_angle=0.0):
    """nerfacc 0.3.3 ray_marching (models/neus.py:156-166,210-220): returns
    packed (ray_indices int32 (n,), t_starts (n, 1), t_ends (n, 1)), ray-major."""
    if sigma_fn is not None and alpha_fn is not None:
        raise ValueError("only one of sigma_fn and alpha_fn")
    rays_o, rays_d = rays_o.float().contiguous(), rays_d.float().contiguous()
    n = rays_o.shape[0]
    if t_min is None or t_max is None:
        if scene_aabb is not None:
            t_min, t_max = ray_aabb_intersect(rays_o, rays_d, scene_aabb)
        else:
            t_min = torch.zeros_like(rays_o[:, 0])
            t_max = torch.full_like(rays_o[:, 0], 1e10)
    t_min, t_max = t_min.reshape(-1).float(), t_max.reshape(-1).float()
    if near_plane is not None:
        t_min = torch.clamp(t_min, min=near_plane) if not torch.is_tensor(near_plane) \
            else torch.maximum(t_min, near_plane.reshape(-1).float())
    if far_plane is not None:
        t_max = torch.clamp(t_max, max=far_plane) if not torch.is_tensor(far_plane) \
            else torch.minimum(t_max, far_plane.reshape(-1).float())
    if stratified:
        t_min = t_min + torch.rand_like(t_min) * render_step_size
    if grid is not None:
        g = dict(roi=grid.roi, res=(grid.res,) * 3, bits=grid.bits, contraction=grid.contraction)
    else:
        g = dict(roi=ops.UNBOUNDED_ROI, res=(1, 1, 1), bits=None)
    ri, t0, t1, offsets, _ = ops.march(rays_o, rays_d, t_min.contiguous(), t_max.contiguous(),
                                       float(render_step_size), cone_angle=float(cone_angle), **g)
    t_starts, t_ends = t0[:, None], t1[:, None]
    if sigma_fn is not None or alpha_fn is not None:
        # the visibility test of nerfacc 0.3.3: drop the samples behind
        # transmittance < early_stop_eps (and those with alpha < alpha_thre)
        if sigma_fn is not None:
            sigmas = sigma_fn(t_starts, t_ends, ri.long())
            alphas = 1.0 - torch.exp(-sigmas.reshape(-1) * (t1 - t0))
        else:
            alphas = alpha_fn(t_starts, t_ends, ri.long()).reshape(-1)
        keep = ops.transmittance_from_alpha(alphas.float(), offsets) >= early_stop_eps
        if alpha_thre > 0:
            keep &= alphas >= alpha_thre
        ri, t_starts, t_ends = ri[keep], t_starts[keep], t_ends[keep]
    return ri, t_starts, t_ends


def render_weight_from_alpha(alphas, packed_info=None, ray_indices=None, n_rays=None,
                             early_stop_eps=1e-4, alpha_thre=0.0):
    """nerfacc 0.3.3 render_weight_from_alpha (models/neus.py:234)."""
    if alpha_thre > 0:
        raise NotImplementedError("alpha_thre > 0 in render_weight_from_alpha")
    offsets = _packed_offsets(packed_info, ray_indices, n_rays)
    w = ops.render_weight_from_alpha(alphas.reshape(-1).float(), offsets, early_stop_eps)
    return w.reshape(alphas.shape)


def render_weight_from_density(t_starts, t_ends, sigmas, packed_info=None, ray_indices=None,
                               n_rays=None, early_stop_eps=1e-4, alpha_thre=0.0):
    """nerfacc 0.3.3 render_weight_from_density (models/neus.py:171)."""
    offsets = _packed_offsets(packed_info, ray_indices, n_rays)
    w = ops.render_weight_from_density(t_starts.reshape(-1, 1).float(), t_ends.reshape(-1, 1).float(),
                                       sigmas.reshape(-1, 1).float(), offsets)
    return w.reshape(sigmas.shape)


def accumulate_along_rays(weights, ray_indices, values=None, n_rays=None):
    """nerfacc 0.3.3 accumulate_along_rays (models/neus.py:235-240): (n_rays, C)."""
    offsets = _offsets(ray_indices, _n_rays(ray_indices, n_rays))
    w = weights.reshape(-1).float()
    v = values.reshape(w.shape[0], -1).float() if values is not None else None
    return ops.accumulate_along_rays(w[:, None], offsets, v)


def _packed_offsets(packed_info, ray_indices, n_rays):
    if packed_info is not None:
        p = packed_info.long()
        return torch.cat([p[:, 0], (p[-1:, 0] + p[-1:, 1])]) if p.numel() else \
            torch.zeros(1, dtype=torch.int64, device=p.device)
    if ray_indices is None:
        raise ValueError("packed_info or ray_indices is required")
    return _offsets(ray_indices, _n_rays(ray_indices, n_rays))


# ---------------------------------------------------------------- installation


def _module(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    m.__doc__ = f"{name} stand-in backed by libangelo_gb.so (angelo_gb.seam)"
    return m


def modules():
    """{name: module} of the stand-ins (tinycudann, nerfacc,
    nerfacc.intersection)."""
    tcnn = _module("tinycudann", Encoding=Encoding, Network=Network,
                   NetworkWithInputEncoding=NetworkWithInputEncoding,
                   free_temporary_memory=free_temporary_memory)
    inter = _module("nerfacc.intersection", ray_aabb_intersect=ray_aabb_intersect)
    nerfacc = _module("nerfacc", ContractionType=ContractionType, OccupancyGrid=OccupancyGrid,
                      ray_marching=ray_marching, render_weight_from_alpha=render_weight_from_alpha,
                      render_weight_from_density=render_weight_from_density,
                      accumulate_along_rays=accumulate_along_rays, intersection=inter,
                      ray_aabb_intersect=ray_aabb_intersect)
    return {"tinycudann": tcnn, "nerfacc": nerfacc, "nerfacc.intersection": inter}


def install():
    """Register the stand-ins in sys.modules (replacing any modules of those
    names) and return them."""
    mods = modules()
    sys.modules.update(mods)
    return mods
