"""Drop-ins for models/network_utils.py: the progressive-band hash grid, the
composite (xyz + grid) encoding, the SH direction encoding and VanillaMLP.

Module and parameter names follow the reference so that state_dicts line up
(``encoding.encoding.params`` is the flat table exactly where tcnn keeps it;
weight-normalised layers expose ``weight_g`` / ``weight_v``)."""
from __future__ import annotations

import math

import torch
import torch.nn as nn
import torch.nn.functional as F

from . import ops
from .config import to_config, to_primitive


class HashGridEncoding(nn.Module):
    """The table behind tcnn.Encoding(otype=HashGrid): ``params`` holds
    n_entries*F values initialised U(-1e-4, 1e-4), level-major."""

    def __init__(self, n_input_dims, config):
        super().__init__()
        assert n_input_dims == 3, "the hash grid encodes 3-D points"
        self.n_input_dims = 3
        self.spec = ops.HashGridSpec(config["n_levels"], config["n_features_per_level"],
                                     config["log2_hashmap_size"], config["base_resolution"],
                                     config["per_level_scale"])
        self.n_output_dims = self.spec.n_output_dims
        self.params = nn.Parameter(torch.empty(self.spec.n_params, dtype=torch.float32)
                                   .uniform_(-1e-4, 1e-4))

    def forward(self, x, active_levels=None, include_xyz=False):
        return ops.hashgrid_encode(x.float(), self.params, self.spec, active_levels, include_xyz)


class ProgressiveBandHashGrid(nn.Module):
    """models/network_utils.py:40-66: hash grid whose levels >= current_level
    are masked to zero; the level grows start_level + (step-start_step) //
    update_steps.  The mask is applied inside the encode kernel (inactive
    levels are neither gathered nor scattered)."""

    def __init__(self, in_channels, config):
        super().__init__()
        config = to_primitive(config)
        self.n_input_dims = in_channels
        self.encoding = HashGridEncoding(in_channels, config)
        self.n_output_dims = self.encoding.n_output_dims
        self.n_level = config["n_levels"]
        self.n_features_per_level = config["n_features_per_level"]
        self.start_level = config["start_level"]
        self.start_step = config["start_step"]
        self.update_steps = config["update_steps"]
        self.current_level = self.start_level
        # the reference's float mask only ever gains ones: track its extent
        self.mask_levels = self.current_level

    @property
    def mask(self):
        m = torch.zeros(self.n_level * self.n_features_per_level)
        m[: self.mask_levels * self.n_features_per_level] = 1.0
        return m

    def forward(self, x, include_xyz=False):
        return self.encoding(x, self.mask_levels, include_xyz)

    def update_step(self, epoch, global_step):
        self.current_level = min(
            self.start_level + max(global_step - self.start_step, 0) // self.update_steps,
            self.n_level)
        self.mask_levels = max(self.mask_levels, self.current_level)


class SphericalHarmonicsEncoding(nn.Module):
    """tcnn.Encoding(otype=SphericalHarmonics, degree=4) on directions given
    in [0,1]^3 (models/texture.py:24-25)."""

    def __init__(self, n_input_dims, config):
        super().__init__()
        if config["degree"] != 4:
            raise NotImplementedError("only degree-4 spherical harmonics are on the hot path")
        self.n_input_dims = n_input_dims
        self.n_output_dims = 16

    def forward(self, d01):
        return ops.sh4_encode(d01.float().contiguous())


class CompositeEncoding(nn.Module):
    """models/network_utils.py:69-80: [x*2-1, encoding(x)] when include_xyz.
    For the hash grid the concatenation is written by the encode kernel."""

    def __init__(self, encoding, include_xyz=False, xyz_scale=2.0, xyz_offset=-1.0):
        super().__init__()
        self.encoding = encoding
        self.include_xyz, self.xyz_scale, self.xyz_offset = include_xyz, xyz_scale, xyz_offset
        self.n_output_dims = int(self.include_xyz) * self.encoding.n_input_dims + \
            self.encoding.n_output_dims

    def forward(self, x, *args):
        if isinstance(self.encoding, ProgressiveBandHashGrid) and self.xyz_scale == 2.0 \
                and self.xyz_offset == -1.0:
            return self.encoding(x, include_xyz=self.include_xyz)
        e = self.encoding(x, *args)
        if not self.include_xyz:
            return e
        return torch.cat([x * self.xyz_scale + self.xyz_offset, e], dim=-1)

    def update_step(self, epoch, global_step):
        if hasattr(self.encoding, "update_step"):
            self.encoding.update_step(epoch, global_step)


def get_encoding(n_input_dims, config):
    """models/network_utils.py:83-93 (the hot-path encoders)."""
    config = to_config(config)
    if config.otype == "ProgressiveBandHashGrid":
        enc = ProgressiveBandHashGrid(n_input_dims, config)
    elif config.otype == "HashGrid":
        cfg = dict(to_primitive(config))
        cfg.setdefault("start_level", cfg["n_levels"])
        cfg.setdefault("start_step", 0)
        cfg.setdefault("update_steps", 1)
        enc = ProgressiveBandHashGrid(n_input_dims, cfg)
    elif config.otype == "SphericalHarmonics":
        enc = SphericalHarmonicsEncoding(n_input_dims, config)
    else:
        raise NotImplementedError(f"encoding {config.otype} is outside the NeuS hot path")
    return CompositeEncoding(enc, include_xyz=config.get("include_xyz", False), xyz_scale=2.0,
                             xyz_offset=-1.0)


class WNLinear(nn.Module):
    """nn.Linear under the reference's nn.utils.weight_norm (dim 0):
    W = weight_g * weight_v / ||weight_v||_row, with the same parameter names."""

    def __init__(self, lin: nn.Linear):
        super().__init__()
        w = lin.weight.detach()
        self.weight_g = nn.Parameter(w.norm(dim=1, keepdim=True).clone())
        self.weight_v = nn.Parameter(w.clone())
        self.bias = nn.Parameter(lin.bias.detach().clone())
        self.in_features, self.out_features = lin.in_features, lin.out_features

    @property
    def weight(self):
        return self.weight_g * self.weight_v / self.weight_v.norm(dim=1, keepdim=True)

    def forward(self, x):
        return F.linear(x, self.weight, self.bias)


def output_activation(name):
    """VanillaMLP's output activation (models/network_utils.py:107,112 through
    models/utils.py get_activation): none, sigmoid, tanh, relu, exp."""
    if name in (None, "none", "None"):
        return lambda x: x
    fns = {"sigmoid": torch.sigmoid, "tanh": torch.tanh, "relu": torch.relu, "exp": torch.exp}
    key = str(name).lower()
    if key not in fns:
        raise NotImplementedError(f"output activation {name!r}")
    return fns[key]


class VanillaMLP(nn.Module):
    """models/network_utils.py:96-140: Linear(+bias) chain, Softplus(beta=100)
    between layers when sphere_init (ReLU otherwise), FP32."""

    def __init__(self, dim_in, dim_out, config):
        super().__init__()
        config = to_primitive(config)
        self.n_neurons, self.n_hidden_layers = config["n_neurons"], config["n_hidden_layers"]
        self.sphere_init = config.get("sphere_init", False)
        self.weight_norm = config.get("weight_norm", False)
        self.sphere_init_radius = config.get("sphere_init_radius", 0.5)
        layers = [self.make_linear(dim_in, self.n_neurons, True, False), self.make_activation()]
        for _ in range(self.n_hidden_layers - 1):
            layers += [self.make_linear(self.n_neurons, self.n_neurons, False, False),
                       self.make_activation()]
        layers += [self.make_linear(self.n_neurons, dim_out, False, True)]
        self.layers = nn.Sequential(*layers)
        self.output_activation = config.get("output_activation", "none")
        self.dim_in, self.dim_out = dim_in, dim_out
        # set by the fused forms: run on the fused tensor-core MLP kernel
        # (ReLU MLPs of the shapes angelo_gb.fused.mlp_supported accepts)
        self.fused = False

    def forward(self, x):
        if self.fused:
            from . import fused
            if fused.mlp_supported(self):
                return fused.mlp_forward(self, x.reshape(-1, self.dim_in)).view(*x.shape[:-1], self.dim_out)
        x = self.layers(x.float())
        return output_activation(self.output_activation)(x)

    def linears(self):
        return [m for m in self.layers if isinstance(m, (nn.Linear, WNLinear))]

    def effective_weights(self):
        """[(W, b)] of every layer after weight normalisation (differentiable)."""
        return [(m.weight, m.bias) for m in self.linears()]

    def make_linear(self, dim_in, dim_out, is_first, is_last):
        layer = nn.Linear(dim_in, dim_out, bias=True)
        with torch.no_grad():
            if self.sphere_init:
                if is_last:
                    layer.bias.fill_(-self.sphere_init_radius)
                    layer.weight.normal_(math.sqrt(math.pi) / math.sqrt(dim_in), 0.0001)
                elif is_first:
                    layer.bias.zero_()
                    layer.weight.zero_()
                    layer.weight[:, :3].normal_(0.0, math.sqrt(2) / math.sqrt(dim_out))
                else:
                    layer.bias.zero_()
                    layer.weight.normal_(0.0, math.sqrt(2) / math.sqrt(dim_out))
            else:
                layer.bias.zero_()
                nn.init.kaiming_uniform_(layer.weight, nonlinearity="relu")
        return WNLinear(layer) if self.weight_norm else layer

    def make_activation(self):
        return nn.Softplus(beta=100) if self.sphere_init else nn.ReLU(inplace=True)


def get_mlp(n_input_dims, n_output_dims, config):
    config = to_config(config)
    if config.otype != "VanillaMLP":
        raise NotImplementedError(f"network {config.otype}: the hot path uses VanillaMLP")
    return VanillaMLP(n_input_dims, n_output_dims, config)
