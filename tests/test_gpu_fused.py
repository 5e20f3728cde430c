"""Parity of the fused kernels (fused VolumeSDF forward/backward) against the
plain path and against the golden vectors of the reference's own code.  The
fused MLP runs on tensor cores in bf16x3 (fp32 accumulation); tolerances are
written per output below."""
import numpy as np
import pytest
import torch

from golden_util import NAMES, load
from test_gpu_neus import build_model, check_against_golden, run_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _geom_pair(g, dev):
    plain = build_model(g, dev, fused=False)
    fused = build_model(g, dev, fused=True)
    plain.update_step(0, g["cfg"]["global_step"])
    fused.update_step(0, g["cfg"]["global_step"])
    return plain.geometry, fused.geometry


@pytest.mark.parametrize("name", NAMES)
def test_fused_volume_sdf_matches_plain(dev, name):
    g = load(name)
    gp, gf = _geom_pair(g, dev)
    r = g["cfg"]["radius"]
    rng = np.random.default_rng(3)
    n = 3000 + 7                      # not a multiple of the 16-sample tile
    pts = torch.from_numpy(rng.uniform(-r, r, (n, 3)).astype(np.float32)).to(dev)
    pts[:4] = torch.tensor([[-r, -r, -r], [r, r, r], [0, 0, 0], [r, 0, -r]], device=dev)
    rd = torch.from_numpy(rng.normal(size=(n, 3)).astype(np.float32)).to(dev)
    gp.curvature_dirs_fn = lambda t: rd
    gf.curvature_dirs_fn = lambda t: rd
    outs = []
    for geo in (gp, gf):
        geo.zero_grad()
        sdf, grad, feat, lap = geo(pts, with_grad=True, with_feature=True, with_laplace=True)
        w = torch.from_numpy(np.random.default_rng(9).normal(size=(n, 8)).astype(np.float32)).to(dev)
        loss = ((sdf * w[:, 0]).sum() + (grad * w[:, 1:4]).sum() +
                (feat[:, :5] * w[:, 3:8]).sum() + (lap[:, 0] * w[:, 0]).sum() * 1e-2)
        loss.backward()
        grads = {k: p.grad.detach().cpu().numpy().copy() for k, p in geo.named_parameters()
                 if p.grad is not None}
        outs.append(([t.detach().cpu().numpy() for t in (sdf, grad, feat, lap)], grads))
    (sp, gp_, fp, lp), grp = outs[0]
    (sf, gf_, ff, lf), grf = outs[1]
    np.testing.assert_allclose(sf, sp, rtol=1e-5, atol=2e-6)
    np.testing.assert_allclose(ff, fp, rtol=1e-5, atol=2e-6)
    eps = gf._finite_difference_eps
    # FD gradient: SDF differences over 2 eps
    np.testing.assert_allclose(gf_, gp_, rtol=1e-4, atol=4e-6 / eps)
    assert np.mean(np.abs(lf - lp)) < 1e-4
    assert set(grf) == set(grp)
    for k in grp:
        ref, got = grp[k], grf[k]
        scale = max(np.abs(ref).max(), 1e-8)
        err = np.abs(got - ref).max() / scale
        assert err < 5e-3, (k, err)


@pytest.mark.parametrize("name", NAMES)
def test_fused_neus_matches_reference(dev, name):
    g = load(name)
    m, out, grads, grads_curv, rep = run_golden(g, dev, fused=True)
    if "occ_mismatch" in rep:
        assert rep["occ_mismatch"] < 1e-4, rep
    check_against_golden(g, out, grads, grads_curv, out_tol=(3e-4, 3e-5), grad_tol=3e-3)


def test_fused_sdf_query_matches_forward_level(dev):
    g = load("neus_dual_grid")
    gp, gf = _geom_pair(g, dev)
    r = g["cfg"]["radius"]
    pts = torch.rand(100000, 3, device=dev) * 2 * r - r
    with torch.no_grad():
        a = gp.forward_level(pts)
        b = gf.forward_level(pts)
    np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-5, atol=2e-6)
