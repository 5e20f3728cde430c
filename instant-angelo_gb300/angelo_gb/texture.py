"""Drop-ins for the radiance networks of models/texture.py: 'volume-radiance'
(:10-36), 'volume-dual-color' (:38-64) and 'volume-dual-colorV3' (:113-149).
The SH direction encoding runs in the library; the MLPs are VanillaMLPs (or
the fused radiance kernel when the model runs fused, see angelo_gb.fused)."""
from __future__ import annotations

import torch
import torch.nn as nn

from . import models
from .config import to_config
from .network_utils import get_encoding, get_mlp


def _activation(name):
    if name is None or name == "none":
        return lambda x: x
    if name == "sigmoid":
        return torch.sigmoid
    raise NotImplementedError(f"color activation {name} is outside the NeuS hot path")


@models.register("volume-radiance")
class VolumeRadiance(nn.Module):
    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        self.n_dir_dims = config.get("n_dir_dims", 3)
        self.n_output_dims = 3
        self.encoding = get_encoding(self.n_dir_dims, config.dir_encoding_config)
        self.n_input_dims = config.input_feature_dim + self.encoding.n_output_dims
        self.network = get_mlp(self.n_input_dims, self.n_output_dims, config.mlp_network_config)
        self.dual = False

    def network_input(self, features, dirs, *args):
        dirs = (dirs + 1.0) / 2.0
        emb = self.encoding(dirs.reshape(-1, self.n_dir_dims))
        return torch.cat([features.reshape(-1, features.shape[-1]), emb]
                         + [a.reshape(-1, a.shape[-1]) for a in args], dim=-1)

    def forward(self, features, dirs, *args):
        inp = self.network_input(features, dirs, *args)
        color = self.network(inp).view(*features.shape[:-1], self.n_output_dims).float()
        if "color_activation" in self.config:
            color = _activation(self.config.color_activation)(color)
        return color

    def update_step(self, epoch, global_step):
        pass

    def regularizations(self, out):
        return {}


@models.register("volume-dual-color")
class VolumeDualColor(VolumeRadiance):
    """Adds sigmoid(features[..., 1:4]) as a base colour (models/texture.py:54-57)."""

    def __init__(self, config):
        super().__init__(config)
        self.dual = True

    def forward(self, features, dirs, *args):
        inp = self.network_input(features, dirs, *args)
        color = self.network(inp).view(*features.shape[:-1], self.n_output_dims).float()
        if "color_activation" in self.config:
            act = _activation(self.config.color_activation)
            color = act(color) + act(features[..., 1:4])
        return color


@models.register("volume-dual-colorV3")
class VolumeDualColorV3(nn.Module):
    """Camera-direction and reflected-direction branches blended by a weight
    MLP (models/texture.py:113-146).  With ``use_ide`` the reflected branch
    encodes (r + 1) / 2 of the reflected direction r with the integrated
    directional encoding of degree ``ide_degree`` and roughness
    sigmoid(feature 5), the reference's use_ide form (models/texture.py:73-99,
    models/utils.py:209-273)."""

    def __init__(self, config):
        super().__init__()
        self.config = config = to_config(config)
        self.n_dir_dims = config.get("n_dir_dims", 3)
        self.n_output_dims = 3
        self.encoding = get_encoding(self.n_dir_dims, config.dir_encoding_config)
        self.n_input_dims = config.input_feature_dim + self.encoding.n_output_dims
        self.use_ide = bool(config.get("use_ide", False))
        if self.use_ide:
            from .ide import IntegratedDirEncoding
            self.ide = IntegratedDirEncoding(int(config.get("ide_degree", 4)))
            n_ref = config.input_feature_dim + self.ide.n_output_dims
        else:
            n_ref = self.n_input_dims
        self.cam_network = get_mlp(self.n_input_dims, 3, config.mlp_network_config)
        self.ref_network = get_mlp(n_ref, 3, config.mlp_network_config)
        # the reference spells this key 'weitht_network_config' (models/texture.py:125)
        wcfg = config.get("weitht_network_config", config.get("weight_network_config"))
        self.weight_network = get_mlp(config.input_feature_dim, 1, wcfg)

    def forward(self, features, viewdirs, normals):
        dirs = (viewdirs + 1.0) / 2.0
        emb = self.encoding(dirs.reshape(-1, self.n_dir_dims))
        vdotn = (-viewdirs * normals).sum(-1, keepdim=True)
        ref = 2 * vdotn * normals + viewdirs
        ref = (ref + 1.0) / 2.0
        if self.use_ide:
            rough = torch.sigmoid(features[..., 5:6]).reshape(-1, 1)
            remb = self.ide(ref.reshape(-1, self.n_dir_dims), rough)
        else:
            remb = self.encoding(ref.reshape(-1, self.n_dir_dims))
        inp = torch.cat([features.reshape(-1, features.shape[-1]),
                         normals.reshape(-1, normals.shape[-1])], dim=-1)
        w = self.weight_network(inp)
        cam = self.cam_network(torch.cat([inp, emb], -1)).view(*features.shape[:-1], 3).float()
        refc = self.ref_network(torch.cat([inp, remb], -1)).view(*features.shape[:-1], 3).float()
        act = _activation(self.config.color_activation)
        return w * act(refc) + (1 - w) * act(cam)

    def update_step(self, epoch, global_step):
        pass

    def regularizations(self, out):
        return {}
