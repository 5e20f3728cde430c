"""The vectorised CPU restatement of the training step (oracle/cpu_step.py,
the bench's timed CPU baseline) against the FP64 oracle it restates
(oracle/neus_fp64.py, itself pinned to the reference's own model code by the
golden vectors): the same outputs and parameter gradients in float64 on the
same marched samples, and the reference's initialisation."""
import math

import numpy as np
import pytest
import torch

from oracle import cpu_step as C
from oracle import neus_fp64 as O


def _cfg():
    h = dict(otype="ProgressiveBandHashGrid", n_levels=8, n_features_per_level=2,
             log2_hashmap_size=12, base_resolution=4, per_level_scale=1.5, include_xyz=True,
             start_level=4, start_step=0, update_steps=100)
    mlp = dict(otype="VanillaMLP", n_neurons=64, n_hidden_layers=2, sphere_init=True,
               sphere_init_radius=0.5, weight_norm=True)
    return dict(radius=0.5, num_samples_per_ray=256, cos_anneal_end=1000,
                variance=dict(init_val=0.3),
                geometry=dict(feature_dim=13, xyz_encoding_config=h, mlp_network_config=mlp),
                texture=dict(name="volume-dual-color", input_feature_dim=13 + 6,
                             mlp_network_config=dict(n_neurons=64, n_hidden_layers=2)))


SYSTEM = dict(loss=dict(lambda_rgb_mse=10.0, lambda_eikonal=0.1, lambda_curvature=5e-4),
              optimizer=dict(args=dict(lr=0.01, betas=[0.9, 0.99], eps=1e-15),
                             params=dict(geometry=dict(lr=0.01), texture=dict(lr=0.01),
                                         variance=dict(lr=0.001))))


def test_reference_init():
    P, lay = C.reference_init(_cfg(), seed=0)
    t = P["geometry.encoding.encoding.encoding.params"]
    assert t.numel() == lay.n_params and float(t.abs().max()) <= 1e-4
    w0 = P["geometry.network.layers.0.weight_v"]
    assert w0.shape == (64, 3 + 16) and float(w0[:, 3:].abs().max()) == 0.0
    assert torch.allclose(P["geometry.network.layers.0.weight_g"], w0.norm(dim=1, keepdim=True))
    w2 = P["geometry.network.layers.4.weight_v"]
    assert w2.shape == (13, 64) and abs(float(w2.mean()) - math.sqrt(math.pi) / 8) < 1e-3
    assert torch.all(P["geometry.network.layers.4.bias"] == -0.5)
    assert P["texture.network.layers.0.weight"].shape == (64, 13 + 6 + 16)
    assert float(P["variance.variance"]) == pytest.approx(0.3)


def test_step_matches_fp64_oracle():
    torch.manual_seed(0)
    step = C.TrainStep(_cfg(), SYSTEM, global_step=250, variance=0.5,
                       occupancy=torch.ones(16 ** 3, dtype=torch.bool), seed=3)
    with torch.no_grad():
        t = step.P["geometry.encoding.encoding.encoding.params"]
        t.copy_(torch.rand(t.shape, generator=torch.Generator().manual_seed(1)) * 0.1 - 0.05)
        w = step.P["geometry.network.layers.0.weight_v"]
        w[:, 3:].copy_(torch.randn(w[:, 3:].shape, generator=torch.Generator().manual_seed(2)) * 0.1)
    g = np.random.default_rng(4)
    n = 24
    eye = g.normal(size=(n, 3))
    eye = 1.5 * eye / np.linalg.norm(eye, axis=1, keepdims=True)
    d = -eye + g.normal(size=(n, 3)) * 0.1
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = torch.tensor(np.concatenate([eye, d], 1), dtype=torch.float32)
    march = step.march(rays)
    S = len(march[2])
    assert S > 200
    rd = torch.randn(S, 3, generator=torch.Generator().manual_seed(5), dtype=torch.float64)
    bg = torch.tensor([0.2, 0.5, 0.7], dtype=torch.float64)
    target = torch.rand(n, 3, generator=torch.Generator().manual_seed(6), dtype=torch.float64)
    outs, grads = [], []
    for fn in (C.neus_forward, lambda *a: O.neus_render(*a, training=True)):
        P = {k: v.detach().double().clone().requires_grad_(True) for k, v in step.P.items()}
        out = fn(rays.double(), P, step.G, step.T, march, rd, step.cos_ratio, bg)
        O.neus_losses(out, target).backward()
        outs.append(out)
        grads.append({k: v.grad for k, v in P.items()})
    a, b = outs
    for k in ("comp_rgb_full", "opacity", "depth", "sdf_samples", "sdf_grad_samples",
              "sdf_laplace_samples", "weights"):
        assert torch.allclose(a[k].reshape(b[k].shape), b[k], rtol=1e-9, atol=1e-12), k
    for k in grads[1]:
        ga, gb = grads[0][k], grads[1][k]
        # summation order differs (one scatter-add of all corners against one
        # per corner; taps whose stencils clamp to one point contribute
        # cancelling terms scaled by normalize()'s 1e12): ~1e-9 of the scale
        assert float((ga - gb).abs().max()) <= 1e-7 * float(gb.abs().max()), k


def test_step_runs_float32():
    step = C.TrainStep(_cfg(), SYSTEM, global_step=250, variance=0.5,
                       occupancy=torch.ones(16 ** 3, dtype=torch.bool), seed=3)
    rays = torch.tensor([[1.5, 0.1, 0.2, -1.0, 0.0, 0.0], [0.1, 1.5, 0.0, 0.0, -1.0, 0.05]],
                        dtype=torch.float32)
    rays[:, 3:] /= rays[:, 3:].norm(dim=1, keepdim=True)
    before = step.P["texture.network.layers.0.weight"].detach().clone()
    dt, n = step.step(rays, torch.rand(2, 3))
    assert n > 100 and dt > 0
    assert not torch.equal(before, step.P["texture.network.layers.0.weight"].detach())
