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
        # with radius < 1 the reference's curvature stencil (shifted in contracted
        # coordinates, clamped to +-r) collapses for part of the box and its
        # gradient is dy / 1e-12 there in both paths: leave it out of the loss
        lw = 1e-2 if r >= 1.0 else 0.0
        loss = ((sdf * w[:, 0]).sum() + (grad * w[:, 1:4]).sum() +
                (feat[:, :5] * w[:, 3:8]).sum() + (lap[:, 0] * w[:, 0]).sum() * lw)
        loss.backward()
        grads = {k: p.grad.detach().cpu().numpy().copy() for k, p in geo.named_parameters()
                 if p.grad is not None}
        outs.append(([t.detach().cpu().numpy() for t in (sdf, grad, feat, lap)], grads))
    (sp, gp_, fp, lp), grp = outs[0]
    (sf, gf_, ff, lf), grf = outs[1]
    # bf16x3 keeps ~2^-18 of each operand: ~1e-5 on an SDF value of order 1
    np.testing.assert_allclose(sf, sp, rtol=1e-4, atol=3e-5)
    np.testing.assert_allclose(ff, fp, rtol=1e-4, atol=3e-5)
    eps = gf._finite_difference_eps
    # FD gradient: SDF differences over 2 eps
    np.testing.assert_allclose(gf_, gp_, rtol=1e-3, atol=6e-5 / eps)
    assert np.mean(np.abs(lf - lp)) < 2e-3
    assert set(grf) == set(grp)
    for k in grp:
        ref, got = grp[k], grf[k]
        scale = max(np.abs(ref).max(), 1e-8)
        err = np.abs(got - ref).max() / scale
        assert err < 1e-2, (k, err)


@pytest.mark.parametrize("name", NAMES)
def test_fused_neus_matches_reference(dev, name):
    g = load(name)
    m, out, grads, grads_curv, rep = run_golden(g, dev, fused=True)
    if "occ_mismatch" in rep:
        assert rep["occ_mismatch"] < 1e-4, rep
    # the curvature gradient of the output bias is zero in exact arithmetic
    # (a constant SDF shift leaves the normals unchanged); its golden value is
    # float32 noise at the 1e-4 floor, so the curvature tolerance is 5e-2
    check_against_golden(g, out, grads, grads_curv, out_tol=(3e-4, 3e-5), grad_tol=3e-3,
                         curv_tol=5e-2)


def test_fused_sdf_query_matches_forward_level(dev):
    g = load("neus_dual_grid")
    gp, gf = _geom_pair(g, dev)
    r = g["cfg"]["radius"]
    pts = torch.rand(100000, 3, device=dev) * 2 * r - r
    with torch.no_grad():
        a = gp.forward_level(pts)
        b = gf.forward_level(pts)
    np.testing.assert_allclose(b.cpu().numpy(), a.cpu().numpy(), rtol=1e-4, atol=3e-5)


def _render_inputs(g, dev):
    """Plain-path per-sample inputs of the radiance and compositing steps for
    the golden rays (march with the golden's jitter)."""
    m = build_model(g, dev, fused=False)
    m.update_step(0, g["cfg"]["global_step"])
    if g["cfg"]["grid_prune"]:
        m.occupancy_grid.bits.copy_(torch.from_numpy(g["occ_bits"].view(np.int32)).to(dev))
    jit = torch.from_numpy(g["jitter"]).to(dev)
    m.stratified_fn = lambda t: jit
    rays = torch.from_numpy(g["rays"]).to(dev)
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    ri, t0, t1, off = m.march_rays(o, d)
    idx = ri.long()
    mid = (t0 + t1) * 0.5
    pos = o[idx] + d[idx] * mid[:, None]
    rd = torch.from_numpy(g["rand_dirs"]).to(dev)
    m.geometry.curvature_dirs_fn = lambda t: rd
    with torch.no_grad():
        sdf, grad, feat, lap = m.geometry(pos, True, True, True)
    return m, o, d, ri, t0, t1, off, sdf.detach(), grad.detach(), feat.detach()


@pytest.mark.parametrize("name", NAMES)
def test_fused_radiance_matches_plain(dev, name):
    """Fused radiance network vs the plain fp32 module, both judged against
    the same module evaluated in float64."""
    from angelo_gb import fused
    from golden_util import oracle_cfgs
    from oracle import neus_fp64 as O
    g = load(name)
    _, T = oracle_cfgs(g)
    m, o, d, ri, t0, t1, off, sdf, grad, feat = _render_inputs(g, dev)
    tex = m.texture
    # rows with a hidden pre-activation within 1e-4 (relative) of a ReLU kink
    # may take either side in bf16x3, fp32 or fp64; they get no loss weight,
    # so every remaining difference is arithmetic
    with torch.no_grad():
        P64 = {"texture." + k: p.detach().double() for k, p in tex.named_parameters()}
        nrm64 = torch.nn.functional.normalize(grad.double(), p=2, dim=-1)
        inp = torch.cat([feat.double(), O.sh4((d[ri.long()].double() + 1.0) / 2.0), nrm64], -1)
        layers = O.mlp_layers(P64, "texture.network", T["n_layers"], False)
        z1 = torch.nn.functional.linear(inp, *layers[0])
        z2 = torch.nn.functional.linear(torch.relu(z1), *layers[1])
        near = ((z1.abs() < 1e-4 * z1.abs().max()).any(1) |
                (z2.abs() < 1e-4 * z2.abs().max()).any(1)).cpu().numpy()
    assert near.mean() < 0.2
    outs = []
    for mode in ("plain", "fused", "fp64"):
        tex.zero_grad()
        dt = torch.float64 if mode == "fp64" else torch.float32
        f_ = feat.clone().to(dt).requires_grad_(True)
        g_ = grad.clone().to(dt).requires_grad_(True)
        if mode == "fused":
            rgb = fused.radiance_forward(tex, f_, g_, ri, d)
            params = dict(tex.named_parameters())
        elif mode == "plain":
            normal = torch.nn.functional.normalize(g_, p=2, dim=-1)
            rgb = tex(f_, d[ri.long()], normal)
            params = dict(tex.named_parameters())
        else:
            # the oracle's float64 texture on the same weights
            params = {k: p.detach().double().requires_grad_(True) for k, p in tex.named_parameters()}
            normal = torch.nn.functional.normalize(g_, p=2, dim=-1)
            rgb = O.texture(f_, d[ri.long()].double(), normal,
                            {"texture." + k: v for k, v in params.items()}, T)
        wn = np.random.default_rng(1).normal(size=tuple(rgb.shape))
        wn[near] = 0.0
        w = torch.from_numpy(wn).to(dev).to(dt)
        (rgb * w).sum().backward()
        outs.append((rgb.detach().double().cpu().numpy(), f_.grad.double().cpu().numpy(),
                     g_.grad.double().cpu().numpy(),
                     {k: p.grad.double().cpu().numpy().copy() for k, p in params.items()
                      if p.grad is not None}))
    (rp, fp, gp, wp), (rf, ff, gf, wf), (r64, f64, g64, w64) = outs
    np.testing.assert_allclose(rf, rp, rtol=1e-4, atol=2e-5)
    np.testing.assert_allclose(rf, r64, rtol=1e-4, atol=2e-5)

    # input gradients per row and weight gradients (sums over all rows), both
    # against fp64; the fp32 module's own error is reported beside
    np.testing.assert_allclose(ff, f64, rtol=1e-3, atol=1e-5 * max(1.0, np.abs(f64).max()))
    np.testing.assert_allclose(gf, g64, rtol=1e-3, atol=1e-4 * max(1.0, np.abs(g64).max()))
    for k in w64:
        scale = max(np.abs(w64[k]).max(), 1e-8)
        e_f = np.abs(wf[k] - w64[k]).max() / scale
        e_p = np.abs(wp[k] - w64[k]).max() / scale
        assert e_f < 2e-3, (k, e_f, e_p)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("inv_s_var", [0.3, 0.8])   # inv_s 20 and 2981 (fp64-gated alpha)
def test_fused_composite_matches_plain(dev, name, inv_s_var):
    from angelo_gb import fused, ops
    F = torch.nn.functional
    g = load(name)
    m, o, d, ri, t0, t1, off, sdf, grad, feat = _render_inputs(g, dev)
    with torch.no_grad():
        m.variance.variance.fill_(inv_s_var)
        normal0 = F.normalize(grad, p=2, dim=-1)
        rgb0 = m.texture(feat, d[ri.long()], normal0).detach()
    bg = torch.tensor([0.3, 0.5, 0.7], device=dev)
    m.background_color = bg
    rng = np.random.default_rng(5)
    R = off.numel() - 1
    gw = {k: torch.from_numpy(rng.normal(size=s).astype(np.float32)).to(dev)
          for k, s in (("op", (R, 1)), ("dep", (R, 1)), ("rgb", (R, 3)), ("n", (R, 3)),
                       ("full", (R, 3)))}
    res = []
    for use_fused in (False, True):
        m.zero_grad()
        s_ = sdf.clone().requires_grad_(True)
        g_ = grad.clone().requires_grad_(True)
        c_ = rgb0.clone().requires_grad_(True)
        if use_fused:
            meta = dict(cos_ratio=m.cos_anneal_ratio, eps=1e-4, gate=fused.FP64_ALPHA_GATE)
            op, dep, comp, cn, full, w = fused._FusedComposite.apply(
                s_, g_, c_, m.variance.variance.view(1), t0, t1, off, d, bg, meta)
        else:
            nrm = F.normalize(g_, p=2, dim=-1)
            alpha = m.get_alpha(s_, nrm, d[ri.long()], (t1 - t0)[:, None])[..., None]
            w = ops.render_weight_from_alpha(alpha, off)[:, None]
            op = ops.accumulate_along_rays(w, off)
            dep = ops.accumulate_along_rays(w, off, ((t0 + t1) / 2)[:, None])
            comp = ops.accumulate_along_rays(w, off, c_)
            cn = F.normalize(ops.accumulate_along_rays(w, off, nrm), p=2, dim=-1)
            cn = torch.where(op > 0.1, cn, torch.zeros_like(cn))
            full = comp + bg[None] * (1.0 - op)
        loss = ((op * gw["op"]).sum() + (dep * gw["dep"]).sum() + (comp * gw["rgb"]).sum() +
                (cn * gw["n"]).sum() + (full * gw["full"]).sum())
        loss.backward()
        res.append(([t.detach().cpu().numpy() for t in (op, dep, comp, cn, full)],
                    [s_.grad.cpu().numpy(), g_.grad.cpu().numpy(), c_.grad.cpu().numpy(),
                     m.variance.variance.grad.cpu().numpy()]))
    (outs_p, grads_p), (outs_f, grads_f) = res
    for a, b in zip(outs_f, outs_p):
        # log-space transmittance vs the sequential product: ~1e-6 relative
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=2e-5)
    for name_, a, b in zip(("sdf", "grad", "rgb", "variance"), grads_f, grads_p):
        scale = max(np.abs(b).max(), 1e-6)
        assert np.abs(a - b).max() / scale < 2e-3, (name_, np.abs(a - b).max() / scale)


def test_fp16_table_form_equals_fp32_table_with_rounded_values(dev):
    """fused_table_dtype 'fp16': the encode gathers from an fp16 copy of the
    fp32 table.  Every gathered value is then exactly its fp16 rounding, so
    the outputs equal, bit for bit, the fp32-table form run on a table that
    holds the rounded values, and so does the table gradient up to the
    order of its atomic additions (the backward never reads the table)."""
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    a = models.make("neus", workloads.model_config("full", fused=True, fused_table_dtype="fp16")).to(dev)
    b = models.make("neus", workloads.model_config("full", fused=True)).to(dev)
    with torch.no_grad():
        p = a.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=torch.Generator().manual_seed(3)) * 0.1 - 0.05).to(dev))
        b.load_state_dict(a.state_dict())
        b.geometry.hashgrid.encoding.params.copy_(p.half().float())
    assert not torch.equal(a.geometry.hashgrid.encoding.params, b.geometry.hashgrid.encoding.params)
    g = torch.Generator().manual_seed(4)
    pts = ((torch.rand(5000, 3, generator=g) - 0.5) * 0.9).to(dev)
    rd = torch.randn(5000, 3, generator=g).to(dev)
    outs, grads = [], []
    for m in (a, b):
        m.update_step(0, 6000)
        m.train()
        m.geometry.curvature_dirs_fn = lambda t: rd
        m.zero_grad()
        sdf, grad, feat, lap = m.geometry(pts, with_grad=True, with_feature=True, with_laplace=True)
        (sdf.square().sum() + grad.sum() + feat.sum() + lap.sum()).backward()
        outs.append((sdf, grad, feat, lap))
        grads.append(m.geometry.hashgrid.encoding.params.grad.clone())
    for x, y in zip(*outs):
        assert torch.equal(x, y)
    torch.testing.assert_close(grads[0], grads[1], rtol=1e-5, atol=1e-9)
