"""Loading helpers for the golden vectors in tests/golden (made by
tests/golden/make_golden.py from the reference's own model code)."""
from __future__ import annotations

import json
import os

import numpy as np
import torch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ("neus_small", "neus_dual_grid")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["cfg"] = json.loads(str(g["config"]))
    return g


def params(g, dtype=torch.float64):
    return {k[len("param/"):]: torch.tensor(v, dtype=dtype) for k, v in g.items()
            if k.startswith("param/")}


def oracle_cfgs(g):
    from oracle import neus_fp64 as O
    c = g["cfg"]
    h = c["hg"]
    lay = O.HashGridLayout(h["n_levels"], h["n_features_per_level"], h["log2_hashmap_size"],
                           h["base_resolution"], h["per_level_scale"])
    G = dict(radius=c["radius"], eps=float(g["eps"]), lay=lay,
             active_levels=O.band_level(h, c["global_step"]),
             n_layers=c["geo"]["n_hidden_layers"] + 1, feature_dim=c["geo"]["feature_dim"],
             hg=h)
    kind = {"volume-radiance": "radiance", "volume-dual-color": "dual"}[c["tex"]["name"]]
    T = dict(kind=kind, n_layers=c["tex"]["n_hidden_layers"] + 1)
    return G, T


def model_config(g, fused=False, **extra):
    """The reference model config the golden was made with (the keys of
    make_golden.model_config), as a plain dict for the drop-in NeuSModel."""
    from golden.make_golden import model_config as mc
    from angelo_gb.config import to_primitive
    cfg = to_primitive(mc(g["cfg"]))
    cfg["fused"] = fused
    cfg.update(extra)
    return cfg
