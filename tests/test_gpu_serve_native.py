"""The library's native server (angelo_serve_*, C ABI): a render through
its graph-captured buckets is bit-identical to the exact-size render of the
same rays with the same kernels (serve.render_exact), with and without the
graph, with the scene box or near/far planes; buckets that overflow their
sample capacity are rendered again at exact size; SDF queries equal
VolumeSDF.forward_level on the fused kernels."""
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


def _model(dev):
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("small", fused=True)).to(dev)
    m.update_step(0, 5000)
    with torch.no_grad():
        g = torch.Generator(device="cpu").manual_seed(1)
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=g) * 0.1 - 0.05).to(dev))
    return m.eval()


def _rays(dev, W, H, eye, seed=0):
    from angelo_gb.serve import RenderRequest, request_rays
    from angelo_gb.scenes import look_at_c2w
    q = RenderRequest(seed, look_at_c2w(eye), W, H)
    return request_rays(q, 0, q.n, dev)


@pytest.mark.parametrize("use_graph", [True, False])
def test_native_render_equals_exact(dev, use_graph):
    from angelo_gb.serve import NativeServer, render_exact
    m = _model(dev)
    ns = NativeServer(m, rays_per_bucket=2048, samples_per_ray=128, points_per_bucket=4096,
                      background=(0.2, 0.4, 0.6), use_graph=use_graph)
    try:
        # 3072, 3700 and 2541 rays: full and partial buckets
        for W, H, eye in ((64, 48, (2.5, 0.3, 0.4)), (100, 37, (-0.8, 1.9, 1.4)),
                          (33, 77, (0.2, -1.1, -2.2))):
            rays = _rays(dev, W, H, eye)
            rgb, op, dep, ovf = ns.render(rays)
            full, op2, dep2 = render_exact(m, rays, ns.bg)
            assert ovf == 0
            assert torch.equal(rgb, full) and torch.equal(op, op2) and torch.equal(dep, dep2)
        assert float(op.max()) > 0.5           # the views see the surface
    finally:
        ns.close()


def test_native_overflowing_buckets_render_exactly(dev):
    from angelo_gb.serve import NativeServer, render_exact
    m = _model(dev)
    ns = NativeServer(m, rays_per_bucket=1024, samples_per_ray=4, points_per_bucket=4096)
    try:
        rays = _rays(dev, 64, 48, (2.5, 0.3, 0.4))
        rgb, op, dep, ovf = ns.render(rays)
        assert ovf >= 1
        full, op2, dep2 = render_exact(m, rays, ns.bg)
        assert torch.equal(rgb, full) and torch.equal(op, op2) and torch.equal(dep, dep2)
    finally:
        ns.close()


def test_native_render_with_planes(dev):
    from angelo_gb.serve import NativeServer, render_exact
    m = _model(dev)
    m.near_plane, m.far_plane = 1.2, 3.5
    ns = NativeServer(m, rays_per_bucket=2048, samples_per_ray=160, points_per_bucket=4096)
    try:
        rays = _rays(dev, 50, 40, (2.5, 0.3, 0.4))
        rgb, op, dep, ovf = ns.render(rays)
        full, op2, dep2 = render_exact(m, rays, ns.bg)
        assert ovf == 0
        assert torch.equal(rgb, full) and torch.equal(op, op2) and torch.equal(dep, dep2)
    finally:
        ns.close()


def test_native_sdf_equals_forward_level(dev):
    from angelo_gb import fused
    from angelo_gb.serve import NativeServer
    m = _model(dev)
    ns = NativeServer(m, rays_per_bucket=256, samples_per_ray=8, points_per_bucket=5000)
    try:
        g = torch.Generator(device="cpu").manual_seed(4)
        pts = (torch.rand(12345, 3, generator=g) * 1.2 - 0.6).to(dev)
        ref = fused.sdf_query(m.geometry, pts)
        out = ns.sdf(pts)
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    finally:
        ns.close()
