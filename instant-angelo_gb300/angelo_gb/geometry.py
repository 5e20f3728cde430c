"""Drop-in for VolumeSDF (models/geometry.py:180-314), registered as
'volume-sdf'.

Two execution forms share the module and its parameters:
  * plain: the reference's algorithm step by step, with the tcnn seam replaced
    by the library's encode kernels and the MLP left to torch (cuBLAS), as
    the reference runs it;
  * fused (config ``fused: true``): one kernel evaluates the 13 hash-grid +
    MLP evaluations of a sample (main point, 6-tap finite-difference stencil,
    6-tap curvature stencil) and a hand-written backward kernel recomputes
    them (see angelo_gb.fused).
"""
from __future__ import annotations

import math

import numpy as np
import torch
import torch.nn as nn
import torch.nn.functional as F

from . import models
from .config import to_config
from .network_utils import get_encoding, get_mlp


def contract_to_unisphere(x, radius):
    """AABB contraction (models/geometry.py:19-21 with models/utils.py:109-114):
    (x - (-r)) / (r - (-r)) * (1 - 0) + 0."""
    return (x - (-radius)) / (radius - (-radius)) * (1 - 0) + 0


def contract_unbounded_sphere(x, radius):
    """UN_BOUNDED_SPHERE contraction (models/geometry.py:22-28): [-r, r]^3 to
    [-1, 1]^3, points beyond the unit sphere to radius 2 - 1/|x|, then
    [-2, 2]^3 to [0, 1]^3 (a select instead of the masked assignment, so that
    no device read is needed)."""
    x = (x - (-radius)) / (radius - (-radius)) * (1 - 0) + 0
    x = x * 2 - 1
    mag = x.norm(dim=-1, keepdim=True)
    x = torch.where(mag > 1, (2 - 1 / mag) * (x / mag), x)
    return x / 4 + 0.5


class _TruncExp(torch.autograd.Function):
    """exp with the backward's argument clamped at 15 (models/utils.py:53-69)."""

    @staticmethod
    def forward(ctx, x):
        x = x.float()
        ctx.save_for_backward(x)
        return torch.exp(x)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        return g * torch.exp(torch.clamp(x, max=15))


def get_activation(name):
    """models/utils.py:72-98 for the activations the NeuS configs use."""
    if name is None or str(name).lower() == "none":
        return lambda x: x
    name = str(name).lower()
    if name == "trunc_exp":
        return _TruncExp.apply
    if name == "sigmoid":
        return torch.sigmoid
    if name == "tanh":
        return torch.tanh
    if name.startswith("+") or name.startswith("-"):
        return lambda x: x + float(name)
    return getattr(F, name)


class EncodingWithNetwork(nn.Module):
    """models/network_utils.py:188-198."""

    def __init__(self, encoding, network):
        super().__init__()
        self.encoding, self.network = encoding, network

    def forward(self, x):
        return self.network(self.encoding(x))

    def update_step(self, epoch, global_step):
        for m in (self.encoding, self.network):
            if hasattr(m, "update_step"):
                m.update_step(epoch, global_step)


@models.register("volume-density")
class VolumeDensity(nn.Module):
    """The learned background's density field (models/geometry.py:152-177):
    unbounded-sphere contraction -> hash grid (+ x*2-1) -> MLP; density =
    activation(out[..., 0] + density_bias), feature = out."""

    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        self.radius = config.radius
        self.n_input_dims = config.get("n_input_dims", 3)
        self.n_output_dims = config.feature_dim
        encoding = get_encoding(self.n_input_dims, config.xyz_encoding_config)
        network = get_mlp(encoding.n_output_dims, self.n_output_dims, config.mlp_network_config)
        # fused form: the MLP on the fused tensor-core kernel (the hash grid
        # runs on this library's encode kernels in both forms)
        network.fused = bool(config.get("fused", False))
        self.encoding_with_network = EncodingWithNetwork(encoding, network)
        self.contraction_type = "unbounded_sphere"

    def _density(self, out):
        density = out[..., 0]
        if "density_activation" in self.config:
            density = get_activation(self.config.density_activation)(
                density + float(self.config.density_bias))
        return density

    def forward(self, points):
        pts = contract_unbounded_sphere(points, self.radius)
        out = self.encoding_with_network(pts.view(-1, self.n_input_dims)).view(
            *pts.shape[:-1], self.n_output_dims).float()
        feature = out
        if "feature_activation" in self.config:
            feature = get_activation(self.config.feature_activation)(feature)
        return self._density(out), feature

    def fused_reuse_ok(self):
        """Whether the fused form can hand the visibility pass's encodings and
        outputs to the training pass (angelo_gb.fused.density_field_reused):
        the MLP on the fused kernel and the encoding the hash grid's own
        [x*2-1, grid] kernel."""
        from . import fused
        from .network_utils import CompositeEncoding, ProgressiveBandHashGrid
        enc, net = self.encoding_with_network.encoding, self.encoding_with_network.network
        return (getattr(net, "fused", False) and fused.mlp_supported(net)
                and isinstance(enc, CompositeEncoding)
                and isinstance(enc.encoding, ProgressiveBandHashGrid)
                and enc.xyz_scale == 2.0 and enc.xyz_offset == -1.0)

    def encode_and_evaluate(self, points):
        """(contracted points, encodings X, MLP output) of world points, the
        pieces forward() composes (no autograd graph is kept when called
        under no_grad)."""
        pts = contract_unbounded_sphere(points, self.radius).view(-1, self.n_input_dims)
        X = self.encoding_with_network.encoding(pts)
        out = self.encoding_with_network.network(X).float()
        return pts, X, out

    def native_visibility_ok(self):
        """Whether the fused form's native visibility test applies: the reuse
        of fused_reuse_ok and the trunc_exp density the kernel computes."""
        return (self.fused_reuse_ok()
                and str(self.config.get("density_activation", "")).lower() == "trunc_exp")

    def evaluate_contracted(self, pts):
        """(encodings X, MLP output) of contracted points."""
        X = self.encoding_with_network.encoding(pts)
        return X, self.encoding_with_network.network(X).float()

    def outputs(self, out):
        """(density, feature) from the MLP output, as forward() forms them."""
        feature = out
        if "feature_activation" in self.config:
            feature = get_activation(self.config.feature_activation)(feature)
        return self._density(out), feature

    def forward_level(self, points):
        pts = contract_unbounded_sphere(points, self.radius)
        out = self.encoding_with_network(pts.reshape(-1, self.n_input_dims)).reshape(
            *pts.shape[:-1], self.n_output_dims)
        return -self._density(out)

    def update_step(self, epoch, global_step):
        self.encoding_with_network.update_step(epoch, global_step)


_FD_DIRS = [[1.0, 0.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, -1.0, 0.0],
            [0.0, 0.0, 1.0], [0.0, 0.0, -1.0]]


@models.register("volume-sdf")
class VolumeSDF(nn.Module):
    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        self.radius = config.radius
        self.n_output_dims = config.feature_dim
        self.encoding = get_encoding(3, config.xyz_encoding_config)
        self.network = get_mlp(self.encoding.n_output_dims, self.n_output_dims,
                               config.mlp_network_config)
        self.grad_type = config.get("grad_type", "finite_difference")
        if self.grad_type != "finite_difference":
            raise NotImplementedError("the hot path uses grad_type='finite_difference'")
        self.finite_difference_eps = config.get("finite_difference_eps", 1e-3)
        self._finite_difference_eps = (self.finite_difference_eps
                                       if isinstance(self.finite_difference_eps, float) else None)
        for k in ("sdf_activation", "feature_activation"):
            if k in config:
                raise NotImplementedError(f"{k} is not used by the NeuS configs of the hot path")
        self.fused = bool(config.get("fused", False))
        self.fused_precision = config.get("fused_precision", "fp32")
        # "fp16": the fused forward reads an fp16 copy of the (fp32) hash table,
        # made once per pass; gradients still accumulate into the fp32 table
        self.fused_table_dtype = config.get("fused_table_dtype", "fp32")
        if self.fused_table_dtype not in ("fp32", "fp16"):
            raise ValueError(f"fused_table_dtype {self.fused_table_dtype!r}: 'fp32' or 'fp16'")
        # torch.randn_like at models/geometry.py:238; replaceable for parity runs
        self.curvature_dirs_fn = torch.randn_like
        self.contraction_type = None

    # ------------------------------------------------------------------ glue
    @property
    def hashgrid(self):
        return self.encoding.encoding

    def field(self, x_c):
        """MLP(encode(x)) for contracted points (N,3) -> (N, feature_dim)."""
        return self.network(self.encoding(x_c.reshape(-1, 3)))

    def forward(self, points, with_grad=True, with_feature=True, with_laplace=False,
                with_auxiliary_feature=False):
        if with_auxiliary_feature:
            raise NotImplementedError("the auxiliary feature belongs to SH-NeuS, outside the path")
        if self.fused:
            from . import fused
            rv = fused.volume_sdf_forward(self, points, with_grad, with_feature, with_laplace)
        else:
            rv = self._forward_plain(points, with_grad, with_feature, with_laplace)
        rv = [v if self.training else v.detach() for v in rv]
        return rv[0] if len(rv) == 1 else rv

    def _forward_plain(self, points, with_grad, with_feature, with_laplace):
        r = self.radius
        with torch.set_grad_enabled(self.training and torch.is_grad_enabled()):
            points_ = points
            pts = contract_to_unisphere(points, r)
            out = self.field(pts).view(*pts.shape[:-1], self.n_output_dims).float()
            sdf = out[..., 0]
            feature = torch.cat([out, pts * 2 - 1], dim=-1)
            grad = None
            if with_grad:
                eps = self._finite_difference_eps
                off = torch.as_tensor(_FD_DIRS, device=points.device) * eps
                pd = (points_[..., None, :] + off.to(points_)).clamp(-r, r)
                sd = self.field(contract_to_unisphere(pd, r))[..., 0].view(*pts.shape[:-1], 6).float()
                grad = 0.5 * (sd[..., 0::2] - sd[..., 1::2]) / eps
            if with_laplace:
                eps = self._finite_difference_eps
                rd = F.normalize(self.curvature_dirs_fn(pts), dim=-1)
                normals = F.normalize(grad, dim=-1)
                tangent = torch.cross(normals, rd, dim=-1)
                # the shift is applied to the contracted points and the result
                # is then clamped and contracted as if it were in world units
                # (models/geometry.py:246,264-265)
                shifted = pts.clone() + tangent * eps
                off = torch.as_tensor(_FD_DIRS, device=points.device) * eps
                psd = (shifted[..., None, :] + off.to(points_)).clamp(-r, r)
                ssd = self.field(contract_to_unisphere(psd, r))[..., 0].view(*pts.shape[:-1], 6)
                ssd = ssd.float()
                gs = 0.5 * (ssd[..., 0::2] - ssd[..., 1::2]) / eps
                ns = F.normalize(gs, dim=-1)
                dot = (normals * ns).sum(dim=-1, keepdim=True)
                laplace = torch.acos(torch.clamp(dot, -1.0 + 1e-6, 1.0 - 1e-6)) / math.pi
        rv = [sdf]
        if with_grad:
            rv.append(grad)
        if with_feature:
            rv.append(feature)
        if with_laplace:
            rv.append(laplace)
        return rv

    def forward_level(self, points):
        """SDF only (models/geometry.py:289-294); fused: one evaluation per point."""
        if self.fused:
            from . import fused
            return fused.sdf_query(self, points)
        pts = contract_to_unisphere(points, self.radius)
        return self.field(pts).view(*pts.shape[:-1], self.n_output_dims)[..., 0]

    def update_step(self, epoch, global_step):
        """models/geometry.py:296-314: band level and progressive FD eps."""
        self.encoding.update_step(epoch, global_step)
        if isinstance(self.finite_difference_eps, float):
            self._finite_difference_eps = self.finite_difference_eps
        elif self.finite_difference_eps == "progressive":
            h = self.config.xyz_encoding_config
            assert h.otype == "ProgressiveBandHashGrid"
            level = min(h.start_level + max(global_step - h.start_step, 0) // h.update_steps,
                        h.n_levels)
            grid_res = h.base_resolution * h.per_level_scale ** (level - 1)
            self._finite_difference_eps = 2 * self.config.radius / grid_res
        else:
            raise ValueError(f"Unknown finite_difference_eps={self.finite_difference_eps}")

    def regularizations(self, out):
        return {}

    # ---------------------------------------------------------- isosurface
    @torch.no_grad()
    def sdf_grid(self, resolution, bounds=None, block_res=256, device="cuda"):
        """The SDF query lattice of MarchingCubeHelper (models/geometry.py:60-113):
        points x_min + i * (2/resolution) per axis over the bounds, evaluated in
        blocks of (block_res+1)^3 lattice points.  Returns the (nx,ny,nz)
        float32 SDF grid on `device` and the axes; the reference triangulates
        -(-sdf) = sdf at the 0.001 level (models/geometry.py:84,101,119,148)."""
        r = self.radius
        bounds = bounds or ((-r, r), (-r, r), (-r, r))
        intv = 2.0 / resolution
        axes = [torch.arange(lo, hi, intv) for lo, hi in bounds]
        # the 1-D axes go to the device once; each block's points are formed there
        axes_d = [a.to(device) for a in axes]
        grid = torch.empty(*[len(a) for a in axes], dtype=torch.float32, device=device)
        for xi in range(0, len(axes[0]), block_res):
            for yi in range(0, len(axes[1]), block_res):
                for zi in range(0, len(axes[2]), block_res):
                    xs = axes_d[0][xi:xi + block_res + 1]
                    ys = axes_d[1][yi:yi + block_res + 1]
                    zs = axes_d[2][zi:zi + block_res + 1]
                    X, Y, Z = torch.meshgrid(xs, ys, zs, indexing="ij")
                    xyz = torch.stack([X, Y, Z], -1)
                    sdf = self.forward_level(xyz.reshape(-1, 3)).reshape(X.shape)
                    grid[xi:xi + len(xs), yi:yi + len(ys), zi:zi + len(zs)] = sdf.float()
        return grid, axes

    @torch.no_grad()
    def isosurface(self):
        """MarchingCubeHelper.forward at threshold 0.001 (models/geometry.py:
        88-113, 144-149): the lattice on the device, triangulated there (one
        mesh, vertices shared across the reference's blocks)."""
        iso = self.config.get("isosurface")
        if iso is None:
            raise NotImplementedError
        from . import mesh
        sdf, axes = self.sdf_grid(int(iso.resolution))
        intv = 2.0 / int(iso.resolution)
        v, f = mesh.marching_cubes(sdf, 0.001, origin=[float(a[0]) for a in axes],
                                   spacing=(intv, intv, intv))
        return {"v_pos": v.cpu(), "t_pos_idx": f.cpu()}
