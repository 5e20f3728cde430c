"""The benchmark and test workloads, written as the reference's own model /
system configuration keys (configs/neuralangelo-colmap_sparse.yaml:16-147).

* small  : plain method, small, FP32 (8 levels x 2^16, base 16, x1.5; 1 hidden
           layer; 1024 rays, 128 uniform samples between 0.5 and 4.5, no grid;
           FD eps 1e-2; sphere scene).
* full   : Neuralangelo sparse training step (16 levels x 2^22, base 32,
           finest 2048, band mask from 4 levels +1 every 500 steps; 128^3
           occupancy grid, step sqrt(3)*2*0.5/512; rays resized toward 2^18
           samples, at most 8192; FD eps annealed 1/32 -> 1/2048; eikonal 0.1,
           curvature 5e-4; 1600x1200 views of a torus/box/sphere union).
* background(): the sparse configs' learned NeRF++ background, merged into
           either model's keys.
"""
from __future__ import annotations

import copy


def _mlp(n_hidden, sphere=False):
    d = dict(otype="VanillaMLP", activation="ReLU", output_activation="none", n_neurons=64,
             n_hidden_layers=n_hidden)
    if sphere:
        d.update(sphere_init=True, sphere_init_radius=0.5, weight_norm=True)
    return d


SMALL_MODEL = dict(
    name="neus", radius=1.0, num_samples_per_ray=128, render_step_size=1.0 / 32,
    near_plane=0.5, far_plane=4.5, grid_prune=False, randomized=True, ray_chunk=2048,
    cos_anneal_end=0, learned_background=False, background_color="random",
    variance=dict(init_val=0.3, modulate=False),
    geometry=dict(name="volume-sdf", radius=1.0, feature_dim=13, grad_type="finite_difference",
                  finite_difference_eps=1e-2, isosurface=dict(method="mc", resolution=64),
                  xyz_encoding_config=dict(otype="ProgressiveBandHashGrid", n_levels=8,
                                           n_features_per_level=2, log2_hashmap_size=16,
                                           base_resolution=16, per_level_scale=1.5,
                                           include_xyz=True, start_level=8, start_step=0,
                                           update_steps=1000),
                  mlp_network_config=_mlp(1, sphere=True)),
    texture=dict(name="volume-radiance", input_feature_dim=13 + 6,
                 dir_encoding_config=dict(otype="SphericalHarmonics", degree=4),
                 mlp_network_config=_mlp(2), color_activation="sigmoid"),
)

FULL_MODEL = dict(
    name="neus", radius=0.5, num_samples_per_ray=512, grid_prune=True, grid_prune_occ_thre=0.001,
    randomized=True, ray_chunk=2048, cos_anneal_end=20000, learned_background=False,
    background_color="random", variance=dict(init_val=0.3, modulate=False),
    geometry=dict(name="volume-sdf", radius=0.5, feature_dim=65, grad_type="finite_difference",
                  finite_difference_eps="progressive",
                  isosurface=dict(method="mc", resolution=512),
                  xyz_encoding_config=dict(otype="ProgressiveBandHashGrid", n_levels=16,
                                           n_features_per_level=2, log2_hashmap_size=22,
                                           base_resolution=32,
                                           per_level_scale=1.3195079107728942, include_xyz=True,
                                           start_level=4, start_step=0, update_steps=500),
                  mlp_network_config=_mlp(2, sphere=True)),
    texture=dict(name="volume-dual-color", input_feature_dim=65 + 6,
                 dir_encoding_config=dict(otype="SphericalHarmonics", degree=4),
                 mlp_network_config=_mlp(2), color_activation="sigmoid"),
)

def background(n_levels=16, log2_hashmap_size=19, base_resolution=32,
               per_level_scale=1.3195079107728942, start_level=4, update_steps=1000,
               radius=0.5):
    """The learned background of the sparse configs
    (configs/neuralangelo-colmap_sparse.yaml:29,80-117): volume-density with
    trunc_exp(x - 1) density and 8 features, volume-radiance on (feature,
    SH4(dir)), 256 samples per ray, 256^3 unbounded-sphere grid."""
    return dict(
        learned_background=True, num_samples_per_ray_bg=256,
        geometry_bg=dict(name="volume-density", radius=radius, feature_dim=8,
                         density_activation="trunc_exp", density_bias=-1, isosurface=None,
                         xyz_encoding_config=dict(otype="ProgressiveBandHashGrid", n_levels=n_levels,
                                                  n_features_per_level=2,
                                                  log2_hashmap_size=log2_hashmap_size,
                                                  base_resolution=base_resolution,
                                                  per_level_scale=per_level_scale, include_xyz=True,
                                                  start_level=start_level, start_step=0,
                                                  update_steps=update_steps),
                         mlp_network_config=_mlp(1)),
        texture_bg=dict(name="volume-radiance", input_feature_dim=8,
                        dir_encoding_config=dict(otype="SphericalHarmonics", degree=4),
                        mlp_network_config=_mlp(2), color_activation="sigmoid"),
    )


SYSTEM = dict(
    loss=dict(lambda_rgb_mse=10.0, lambda_eikonal=0.1, lambda_curvature=5e-4),
    optimizer=dict(name="AdamW", args=dict(lr=0.01, betas=[0.9, 0.99], eps=1e-15),
                   params=dict(geometry=dict(lr=0.01), texture=dict(lr=0.01),
                               geometry_bg=dict(lr=0.01), texture_bg=dict(lr=0.01),
                               variance=dict(lr=0.001))),
)


def model_config(name, fused=False, **overrides):
    cfg = copy.deepcopy({"small": SMALL_MODEL, "full": FULL_MODEL}[name])
    cfg["fused"] = fused
    cfg.update(overrides)
    return cfg
