"""End-to-end parity of the drop-in NeuSModel on the GPU against the golden
vectors produced by the reference's own model code (tests/golden): same
parameters, same random draws, same occupancy grid; outputs and parameter
gradients of the training losses within the tolerances written below."""
import numpy as np
import pytest
import torch

from golden_util import NAMES, load, model_config

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def build_model(g, dev, fused=False, **extra):
    from angelo_gb import models
    m = models.make("neus", model_config(g, fused=fused, **extra)).to(dev)
    sd = m.state_dict()
    for k in sd:
        if "param/" + k in g:
            sd[k] = torch.from_numpy(g["param/" + k]).to(dev)
    m.load_state_dict(sd)
    m.train()
    return m


def run_golden(g, dev, fused=False, check_occupancy=True, **extra):
    c = g["cfg"]
    m = build_model(g, dev, fused=fused, **extra)
    report = {}
    if c["grid_prune"]:
        grid = m.occupancy_grid
        seed = c["occ_seed"]
        grid.jitter_fn = lambda t: torch.from_numpy(
            np.random.default_rng(seed).random(tuple(t.shape), dtype=np.float32)).to(t.device)
        m.update_step(0, c["global_step"])
        ours = grid.binary.cpu().numpy().reshape(-1)
        ref = np.unpackbits(g["occ_bits"], bitorder="little").astype(bool)
        report["occ_mismatch"] = float(np.mean(ours != ref))
        sel = g["occ_sample_cells"]
        report["occ_value_err"] = float(np.abs(grid.occs.cpu().numpy()[sel] -
                                               g["occ_sample_values"]).max())
        # render on the reference's own grid so both march the same samples
        grid.bits.copy_(torch.from_numpy(g["occ_bits"].view(np.int32)).to(dev))
    else:
        m.update_step(0, c["global_step"])
    jit = torch.from_numpy(g["jitter"]).to(dev)
    m.stratified_fn = lambda t: jit
    rd = torch.from_numpy(g["rand_dirs"]).to(dev)
    m.geometry.curvature_dirs_fn = lambda t: rd
    m.background_color = torch.from_numpy(g["background"]).to(dev)
    rays = torch.from_numpy(g["rays"]).to(dev)
    out = m.forward_(rays)
    target = torch.from_numpy(g["target"]).to(dev)
    valid = out["rays_valid_full"][..., 0]
    l_main = (torch.nn.functional.mse_loss(out["comp_rgb_full"][valid], target[valid]) * 10.0
              + ((torch.linalg.norm(out["sdf_grad_samples"], ord=2, dim=-1) - 1.0) ** 2).mean()
              * 0.1)
    l_curv = out["sdf_laplace_samples"].abs().mean() * 5e-4
    l_main.backward(retain_graph=True)
    grads = {k: p.grad.detach().cpu().numpy().copy() for k, p in m.named_parameters()
             if p.grad is not None}
    m.zero_grad()
    l_curv.backward()
    grads_curv = {k: p.grad.detach().cpu().numpy().copy() for k, p in m.named_parameters()
                  if p.grad is not None}
    return m, out, grads, grads_curv, report


def check_against_golden(g, out, grads, grads_curv, out_tol=(2e-4, 2e-5), grad_tol=2e-3,
                         fd_tol=2e-3, curv_tol=2e-2):
    np.testing.assert_array_equal(out["ray_indices"].cpu().numpy(), g["out/ray_indices"])
    for k in ("comp_rgb", "opacity", "depth", "comp_rgb_full", "sdf_samples", "weights",
              "points", "intervals"):
        np.testing.assert_allclose(out[k].detach().cpu().numpy().reshape(g["out/" + k].shape),
                                   g["out/" + k], rtol=out_tol[0], atol=out_tol[1], err_msg=k)
    np.testing.assert_allclose(out["sdf_grad_samples"].detach().cpu().numpy(),
                               g["out/sdf_grad_samples"], rtol=fd_tol, atol=fd_tol)
    np.testing.assert_allclose(out["comp_normal"].detach().cpu().numpy(), g["out/comp_normal"],
                               rtol=1e-3, atol=1e-3)
    lap = out["sdf_laplace_samples"].detach().cpu().numpy()
    assert np.mean(np.abs(lap - g["out/sdf_laplace_samples"])) < 2e-3
    gmax = max(np.abs(g[k]).max() for k in g if k.startswith("grad/"))
    for k, v in grads.items():
        ref = g.get("grad/" + k)
        if ref is None:
            continue
        scale = max(np.abs(ref).max(), 1e-4 * gmax)
        err = np.abs(v.reshape(ref.shape) - ref).max() / scale
        assert err < grad_tol, (k, err)
    if g["cfg"]["radius"] >= 1.0:
        gmax = max(np.abs(g[k]).max() for k in g if k.startswith("grad_curv/"))
        for k, v in grads_curv.items():
            ref = g.get("grad_curv/" + k)
            if ref is None:
                continue
            scale = max(np.abs(ref).max(), 1e-4 * gmax)
            err = np.abs(v.reshape(ref.shape) - ref).max() / scale
            assert err < curv_tol, ("curv", k, err)


@pytest.mark.parametrize("name", NAMES)
def test_plain_neus_matches_reference(dev, name):
    g = load(name)
    m, out, grads, grads_curv, rep = run_golden(g, dev)
    if "occ_mismatch" in rep:
        assert rep["occ_mismatch"] < 1e-4, rep
        assert rep["occ_value_err"] < 1e-5, rep
    check_against_golden(g, out, grads, grads_curv)


def test_plain_neus_eval_chunks(dev):
    """Eval renders in ray chunks moved to the CPU (models/neus.py:288-289);
    the result equals the training-mode forward without stratification."""
    g = load("neus_small")
    m = build_model(g, dev)
    m.update_step(0, g["cfg"]["global_step"])
    m.background_color = torch.ones(3, device=dev)
    rd = torch.from_numpy(g["rand_dirs"]).to(dev)
    rays = torch.from_numpy(g["rays"]).to(dev)
    m.eval()
    m.geometry.curvature_dirs_fn = torch.randn_like
    m.config.ray_chunk = 7
    with torch.no_grad():
        out = m(rays)
    assert out["comp_rgb_full"].device.type == "cpu" and out["comp_rgb_full"].shape == (48, 3)
    m.config.ray_chunk = 4096
    with torch.no_grad():
        out2 = m(rays)
    np.testing.assert_allclose(out["comp_rgb_full"].numpy(), out2["comp_rgb_full"].numpy(),
                               rtol=1e-5, atol=1e-6)
