"""Generate the golden vectors in this directory by running the reference's own
model code (models/neus.py, models/geometry.py, models/texture.py,
models/network_utils.py) on the CPU through ``oracle.ref_harness``.

Run from the repository root, in a container that has the reference tree:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /root/reference

Each ``.npz`` holds the configuration (JSON), the parameters (state_dict keys of
the reference module tree), the inputs, every random draw the reference makes
(stratified jitter, curvature directions, occupancy jitter seed), and the outputs
and parameter gradients of one training forward/backward.  The reference runs in
float32 exactly as it does in training (VanillaMLP casts to float32,
models/network_utils.py:109-111).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref_harness as H  # noqa: E402

CONFIGS = {
    # config-1 architecture (1 hidden layer, feature_dim 13, VolumeRadiance), small table
    "neus_small": dict(
        radius=1.0, num_samples_per_ray=64, grid_prune=False, randomized=True,
        cos_anneal_end=20000, global_step=5000, n_rays=48, seed=1,
        hg=dict(otype="ProgressiveBandHashGrid", n_levels=8, n_features_per_level=2,
                log2_hashmap_size=12, base_resolution=16, per_level_scale=1.5, include_xyz=True,
                start_level=4, start_step=0, update_steps=2000),
        geo=dict(feature_dim=13, n_hidden_layers=1),
        tex=dict(name="volume-radiance", n_hidden_layers=2),
    ),
    # config-2 architecture (2 hidden layers, feature_dim 65, VolumeDualColor),
    # occupancy grid on, small table
    "neus_dual_grid": dict(
        radius=0.5, num_samples_per_ray=96, grid_prune=True, randomized=True,
        cos_anneal_end=0, global_step=0, n_rays=40, seed=2, occ_seed=7,
        hg=dict(otype="ProgressiveBandHashGrid", n_levels=16, n_features_per_level=2,
                log2_hashmap_size=10, base_resolution=4, per_level_scale=1.3195079107728942,
                include_xyz=True, start_level=4, start_step=0, update_steps=500),
        geo=dict(feature_dim=65, n_hidden_layers=2),
        tex=dict(name="volume-dual-color", n_hidden_layers=2),
    ),
}


def model_config(c):
    A = H.AttrDict.wrap
    geo = dict(name="volume-sdf", radius=c["radius"], feature_dim=c["geo"]["feature_dim"],
               grad_type="finite_difference", finite_difference_eps="progressive",
               isosurface=None, xyz_encoding_config=c["hg"],
               mlp_network_config=dict(otype="VanillaMLP", activation="ReLU",
                                       output_activation="none", n_neurons=64,
                                       n_hidden_layers=c["geo"]["n_hidden_layers"],
                                       sphere_init=True, sphere_init_radius=0.5,
                                       weight_norm=True))
    tex = dict(name=c["tex"]["name"], input_feature_dim=c["geo"]["feature_dim"] + 6,
               dir_encoding_config=dict(otype="SphericalHarmonics", degree=4),
               mlp_network_config=dict(otype="VanillaMLP", activation="ReLU",
                                       output_activation="none", n_neurons=64,
                                       n_hidden_layers=c["tex"]["n_hidden_layers"]),
               color_activation="sigmoid")
    return A(dict(name="neus", radius=c["radius"], num_samples_per_ray=c["num_samples_per_ray"],
                  grid_prune=c["grid_prune"], grid_prune_occ_thre=0.001, randomized=c["randomized"],
                  ray_chunk=2048, cos_anneal_end=c["cos_anneal_end"], learned_background=False,
                  background_color="random", variance=dict(init_val=0.3, modulate=False),
                  geometry=geo, texture=tex))


def camera_rays(n, radius_cam, seed):
    """Origins on a sphere of radius ``radius_cam`` looking at the origin, with
    directions perturbed inside a 64-degree cone; normalised."""
    g = np.random.default_rng(seed)
    o = g.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * radius_cam
    fwd = -o / np.linalg.norm(o, axis=1, keepdims=True)
    jitter = g.uniform(-0.25, 0.25, size=(n, 3))
    d = fwd + jitter
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def run(name, c, models):
    torch.manual_seed(c["seed"])
    cfg = model_config(c)
    model = models.make("neus", cfg)
    model.train()
    # Move away from the sphere initialisation (whose zero weights on the hash
    # features make the table gradient vanish) to a partly trained state.
    with torch.no_grad():
        gen = torch.Generator().manual_seed(c["seed"] + 50)
        table = model.geometry.encoding.encoding.encoding.params
        table.copy_(torch.rand(table.shape, generator=gen) * 0.2 - 0.1)
        v0 = model.geometry.network.layers[0].weight_v
        v0[:, 3:] = torch.randn(v0[:, 3:].shape, generator=gen) * 0.05
    if c["grid_prune"]:
        occ_seed = c["occ_seed"]
        grid = model.occupancy_grid
        orig = torch.rand_like

        def seeded_rand_like(t, dtype=None, **kw):
            if t.shape == grid.grid_coords.shape:
                g = np.random.default_rng(occ_seed)
                return torch.from_numpy(g.random(t.shape, dtype=np.float32))
            return orig(t, dtype=dtype, **kw)
        torch.rand_like = seeded_rand_like
        model.update_step(0, c["global_step"])
        torch.rand_like = orig
    else:
        model.update_step(0, c["global_step"])
    rays = torch.from_numpy(camera_rays(c["n_rays"], 2.5 * c["radius"], c["seed"]))
    bg = torch.tensor([0.3, 0.5, 0.7])
    model.background_color = bg
    captured = {}
    orig_randn = torch.randn_like

    def rec_randn(t, **kw):
        v = orig_randn(t, **kw)
        captured["rand_dirs"] = v.detach().numpy().copy()
        return v
    torch.randn_like = rec_randn
    out = model.forward_(rays)
    torch.randn_like = orig_randn
    g = np.random.default_rng(c["seed"] + 100)
    target = torch.from_numpy(g.random((c["n_rays"], 3), dtype=np.float32))
    valid = out["rays_valid_full"][..., 0]
    # main loss (rgb MSE + eikonal, systems/neus.py:130-140) and the curvature
    # loss (systems/neus.py:155-159) are differentiated separately: the
    # curvature gradient is ill-conditioned where the shifted stencil collapses
    # under the clamp (models/geometry.py:264-265) and is only compared where
    # the scene radius keeps the stencil inside the box.
    loss_main = (torch.nn.functional.mse_loss(out["comp_rgb_full"][valid], target[valid]) * 10.0
                 + ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean()
                 * 0.1)
    loss_curv = out["sdf_laplace_samples"].abs().mean() * 5e-4
    loss = loss_main + loss_curv
    loss_main.backward(retain_graph=True)
    grads_main = {k: p.grad.detach().numpy().copy() for k, p in model.named_parameters()
                  if p.grad is not None}
    model.zero_grad()
    loss_curv.backward()
    grads_curv = {k: p.grad.detach().numpy().copy() for k, p in model.named_parameters()
                  if p.grad is not None}
    rec = dict(H._MARCH_RECORD)
    blob = {"config": np.array(json.dumps(c)), "rays": rays.numpy(), "background": bg.numpy(),
            "target": target.numpy(), "loss": np.array(loss.item(), np.float32),
            "rand_dirs": captured["rand_dirs"], "jitter": rec["jitter"],
            "t_min": rec["t_min"], "t_max": rec["t_max"], "offsets": rec["offsets"],
            "eps": np.array(model.geometry._finite_difference_eps, np.float64),
            "cos_anneal_ratio": np.array(model.cos_anneal_ratio, np.float64)}
    for k, v in model.state_dict().items():
        if k.startswith("occupancy_grid."):
            continue
        blob["param/" + k] = v.detach().numpy()
    for k, v in grads_main.items():
        blob["grad/" + k] = v
    for k, v in grads_curv.items():
        blob["grad_curv/" + k] = v
    for k in ("comp_rgb", "comp_normal", "opacity", "depth", "comp_rgb_full", "sdf_samples",
              "sdf_grad_samples", "sdf_laplace_samples", "weights", "points", "intervals",
              "ray_indices"):
        blob["out/" + k] = out[k].detach().numpy()
    if c["grid_prune"]:
        grid = model.occupancy_grid
        blob["occ_bits"] = np.packbits(grid.binary.numpy().reshape(-1), bitorder="little")
        sel = np.random.default_rng(5).choice(grid.num_cells, 4096, replace=False)
        blob["occ_sample_cells"] = sel.astype(np.int64)
        blob["occ_sample_values"] = grid.occs.numpy()[sel]
        blob["occ_mean"] = np.array(grid.occs.mean().item(), np.float64)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **blob)
    print(f"{name}: {len(out['ray_indices'])} samples, loss {loss.item():.6f} -> {path}")


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <path of the Instant-angelo source tree>")
    ref = sys.argv[1]
    models = H.install(ref)
    for name, c in CONFIGS.items():
        run(name, c, models)


if __name__ == "__main__":
    main()
