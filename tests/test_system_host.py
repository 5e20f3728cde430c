"""Host logic of the training step (angelo_gb.system) that needs no GPU: the
loss terms the native step computes against the terms a reference loss
config asks for (systems/neus.py:130-196).  A config that weights a term the
step does not compute is refused, not trained with a different objective."""
import pytest
import torch

from angelo_gb import system

# the loss section of the reference's masked sparse config
# (configs/neuralangelo-colmap_sparse-wmask.yaml, system.loss)
WMASK_LOSS = dict(lambda_sdf_l1=[0, 1, 0, 20000], lambda_normal=0.0, lambda_rgb_mse=10.0,
                  lambda_rgb_l1=0.0, lambda_mask=1.0, lambda_eikonal=0.1,
                  lambda_curvature=[0, 0, 5e-2, 5000], lambda_sparsity=0.0,
                  lambda_distortion=0.0, lambda_distortion_bg=0.0, lambda_opaque=0.0)


def test_supported_terms_pass():
    cfg = dict(lambda_rgb_mse=10.0, lambda_eikonal=0.1, lambda_curvature=[0, 0, 5e-4, 5000],
               lambda_rgb_l1=0.0, lambda_sparsity=0.0, lambda_sdf_l1=0.0)
    for step in (0, 100, 30000):
        assert system.unsupported_loss_terms(cfg, step) == {}


def test_wmask_config_reports_mask_and_sdf_l1():
    bad = system.unsupported_loss_terms(WMASK_LOSS, 0)
    assert set(bad) == {"lambda_mask", "lambda_sdf_l1"}
    # the sdf_l1 schedule [0, 1, 0, 20000] reaches 0 at step 20000; the mask
    # term counts only with masked data
    assert set(system.unsupported_loss_terms(WMASK_LOSS, 20000)) == {"lambda_mask"}
    assert system.unsupported_loss_terms(WMASK_LOSS, 20000, has_mask=False) == {}


def test_trainer_refuses_wmask_config():
    model = torch.nn.Module()
    with pytest.raises(NotImplementedError, match="lambda_mask"):
        system.NeuSTrainer(model, {"loss": WMASK_LOSS})


def test_background_fused_routing():
    """Which background modules run on the fused kernels (host logic, CPU):
    the sparse configs' VolumeRadiance texture and ReLU density MLP do; a
    texture with another input, activation or depth does not."""
    from angelo_gb import models, neus, workloads
    cfg = workloads.background(n_levels=8, log2_hashmap_size=12, base_resolution=16,
                               per_level_scale=1.5, start_level=8, radius=1.0)
    tex = models.make(cfg["texture_bg"]["name"], cfg["texture_bg"])
    assert neus.fused_radiance_bg(tex)
    for change in ({"color_activation": "none"},
                   {"mlp_network_config": {**cfg["texture_bg"]["mlp_network_config"], "n_hidden_layers": 1}},
                   {"input_feature_dim": 40}):
        assert not neus.fused_radiance_bg(models.make("volume-radiance", {**cfg["texture_bg"], **change}))
    geo_cfg = dict(cfg["geometry_bg"])
    assert not models.make(geo_cfg["name"], geo_cfg).fused_reuse_ok()
    geo = models.make(geo_cfg["name"], {**geo_cfg, "fused": True})
    assert geo.encoding_with_network.network.fused and geo.fused_reuse_ok()
