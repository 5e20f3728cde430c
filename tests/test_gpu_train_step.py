"""The step's small native parts against their PyTorch fp32 statements:
weight normalisation of the geometry MLP (nn.utils.weight_norm, dim 0,
models/network_utils.py:132-133) forward and backward, and the seeded loss
(systems/neus.py:130-159) forward and backward."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _wn_torch(v, g):
    return g * v / v.norm(dim=1, keepdim=True)


@pytest.mark.parametrize("shapes", [[(64, 35), (64, 64), (65, 64)], [(64, 19), (13, 64)], [(1, 1)]])
def test_weight_norm_matches_torch(dev, shapes):
    from angelo_gb.fused import _WeightNorm
    gen = torch.Generator(device=dev).manual_seed(len(shapes))
    vs = [torch.randn(*s, device=dev, generator=gen).requires_grad_() for s in shapes]
    gs = [(torch.rand(s[0], 1, device=dev, generator=gen) + 0.5).requires_grad_() for s in shapes]
    vg = []
    for v, g in zip(vs, gs):
        vg += [v, g]
    ws = _WeightNorm.apply(*vg)
    ref = [_wn_torch(v, g) for v, g in zip(vs, gs)]
    for w, r in zip(ws, ref):
        torch.testing.assert_close(w, r, rtol=1e-6, atol=1e-7)
    dws = [torch.randn_like(w) for w in ws]
    got = torch.autograd.grad(ws, vg, dws)
    exp = torch.autograd.grad(ref, vg, dws)
    for a, b in zip(got, exp):
        torch.testing.assert_close(a, b, rtol=2e-5, atol=1e-6)


def _inputs(dev, R, S, n_valid, seed):
    gen = torch.Generator(device=dev).manual_seed(seed)
    c = torch.rand(R, 3, device=dev, generator=gen).requires_grad_()
    t = torch.rand(R, 3, device=dev, generator=gen)
    valid = torch.zeros(R, 1, dtype=torch.bool, device=dev)
    valid[torch.randperm(R, device=dev, generator=gen)[:n_valid]] = True
    g = (torch.randn(S, 3, device=dev, generator=gen) * 0.7).requires_grad_()
    with torch.no_grad():
        g[:3] = 0.0   # zero-norm gradients: the norm's backward is 0 there
    lap = torch.randn(S, 1, device=dev, generator=gen)
    with torch.no_grad():
        lap[:5] = 0.0
    lap.requires_grad_()
    return {"comp_rgb_full": c, "rays_valid_full": valid, "sdf_grad_samples": g,
            "sdf_laplace_samples": lap}, t


@pytest.mark.parametrize("R,S,n_valid,w_curv", [(7000, 290000, 6500, 5e-4), (33, 257, 33, 0.0),
                                                (1000, 5000, 1, 1e-3)])
def test_loss_matches_torch(dev, R, S, n_valid, w_curv):
    from angelo_gb.system import fused_loss_terms, loss_terms
    out, t = _inputs(dev, R, S, n_valid, R + S)
    kw = dict(eikonal_weight=0.1, curvature_weight=w_curv, rgb_mse_weight=10.0)
    tot, terms = fused_loss_terms(out, t, **kw)
    rtot, rterms = loss_terms(out, t, **kw)
    torch.testing.assert_close(tot, rtot, rtol=1e-5, atol=0.0)
    for k in rterms:
        torch.testing.assert_close(terms[k], rterms[k], rtol=1e-5, atol=0.0)
    xs = [out["comp_rgb_full"], out["sdf_grad_samples"], out["sdf_laplace_samples"]]
    got = torch.autograd.grad(tot * 1.7, xs, allow_unused=True)
    exp = torch.autograd.grad(rtot * 1.7, xs, allow_unused=True)
    for a, b in zip(got, exp):
        if b is None:
            assert a is None or float(a.abs().max()) == 0.0
            continue
        # (||g|| - 1) cancels near unit norm: absolute tolerance on the
        # gradient's scale for those elements
        torch.testing.assert_close(a, b, rtol=1e-5, atol=1e-6 * float(b.abs().max()))


def test_loss_without_valid_rays_is_nan_and_deterministic(dev):
    from angelo_gb.system import fused_loss_terms
    out, t = _inputs(dev, 64, 1000, 0, 3)
    tot, terms = fused_loss_terms(out, t)
    assert torch.isnan(terms["rgb_mse"]) and torch.isnan(tot)
    out, t = _inputs(dev, 5000, 100000, 4000, 4)
    a = fused_loss_terms(out, t)[0]
    b = fused_loss_terms(out, t)[0]
    assert float(a) == float(b)
