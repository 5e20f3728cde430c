"""The serving loop (angelo_gb.serve): a render request gives the same
result alone and mixed with other renders and SDF grids (bucket composition
does not change per-ray arithmetic), equal to the exact-size render of the
same rays; a bucket that overflows its sample capacity is re-rendered
exactly; SDF grids equal VolumeSDF.forward_level on the lattice."""
import numpy as np
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


def _model(dev, fused=True):
    from angelo_gb import models, workloads
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("small", fused=fused)).to(dev)
    m.update_step(0, 5000)
    with torch.no_grad():
        g = torch.Generator(device="cpu").manual_seed(1)
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=g) * 0.1 - 0.05).to(dev))
    return m.eval()


def _requests(dev):
    from angelo_gb.serve import RenderRequest, SdfGridRequest
    from angelo_gb.scenes import look_at_c2w
    c = [look_at_c2w(e) for e in ((2.5, 0.3, 0.4), (-0.8, 1.9, 1.4), (0.2, -1.1, -2.2))]
    return (RenderRequest(0, c[0], 64, 48), RenderRequest(1, c[1], 100, 37),
            SdfGridRequest(2, 24), RenderRequest(3, c[2], 33, 77))


def test_render_same_alone_and_in_mix(dev):
    from angelo_gb.serve import RenderRequest, Server, render_exact, request_rays
    m = _model(dev)
    srv = Server(m, ray_bucket=2048, max_samples_per_ray=128, point_bucket=1 << 12,
                 hbm_reserve=1 << 30)
    a, b, grid, c = _requests(dev)
    alone = RenderRequest(0, a.c2w, a.W, a.H)
    srv.run([alone], realtime=False)
    srv.run([b, grid, a, c], realtime=False)
    assert torch.equal(a.rgb, alone.rgb) and torch.equal(a.opacity, alone.opacity)
    assert torch.equal(a.depth, alone.depth)
    for q in (a, b, c):
        full, op, dep = render_exact(m, request_rays(q, 0, q.n, dev), srv.bg)
        assert torch.equal(q.rgb, full), q.rid
        assert torch.equal(q.opacity, op) and torch.equal(q.depth, dep)
        assert q.done is not None and q.done >= q.arrival
    assert srv.overflows == 0
    assert float(a.opacity.max()) > 0.5      # the view sees the surface
    assert len(srv.rbs) == 2 and srv.buckets > 2


def test_single_render_stream_gives_the_same_result(dev):
    from angelo_gb.serve import RenderRequest, Server
    m = _model(dev)
    a, b, grid, c = _requests(dev)
    outs = []
    for streams in (1, 2):
        srv = Server(m, ray_bucket=2048, max_samples_per_ray=128, point_bucket=1 << 12,
                     hbm_reserve=1 << 30, render_streams=streams)
        qs = [RenderRequest(q.rid, q.c2w, q.W, q.H) for q in (a, b, c)]
        srv.run(qs, realtime=False)
        outs.append(qs)
    for q1, q2 in zip(*outs):
        assert torch.equal(q1.rgb, q2.rgb) and torch.equal(q1.depth, q2.depth)


def test_overflowing_bucket_is_rendered_exactly(dev):
    from angelo_gb.serve import RenderRequest, Server, render_exact, request_rays
    m = _model(dev)
    a = _requests(dev)[0]
    srv = Server(m, ray_bucket=1024, max_samples_per_ray=16, point_bucket=1 << 12,
                 hbm_reserve=1 << 30)
    q = RenderRequest(0, a.c2w, a.W, a.H)
    srv.run([q], realtime=False)
    assert srv.overflows > 0
    # each bucket's own compositing walked only the samples the fill kept:
    # its offsets never pass the capacity, and those of an overflowed replay
    # end at it
    ends = []
    for rb in srv.rbs:
        off = rb.offsets.cpu()
        assert int(off[-1]) <= rb.cap and bool((off[1:] >= off[:-1]).all())
        ends.append(int(off[-1]) == rb.cap)
    assert any(ends)
    full, op, dep = render_exact(m, request_rays(q, 0, q.n, dev), srv.bg)
    assert torch.equal(q.rgb, full)


def test_offsets_clamp(dev):
    from angelo_gb import _lib, ops
    off = torch.tensor([0, 5, 9, 20, 31, 40], device=dev, dtype=torch.int64)
    _lib.call("angelo_offsets_clamp", ops._p(off), off.numel() - 1, 19, ops._s(dev))
    assert off.cpu().tolist() == [0, 5, 9, 19, 19, 19]


def test_sdf_grid_matches_forward_level(dev):
    from angelo_gb.serve import SdfGridRequest, Server, request_points
    m = _model(dev)
    plain = _model(dev, fused=False)
    srv = Server(m, ray_bucket=1024, max_samples_per_ray=128, point_bucket=5000,
                 hbm_reserve=1 << 30)
    q = SdfGridRequest(0, 33)                 # 35937 points: 8 buckets, the last partial
    srv.run([q], realtime=False)
    pts = request_points(q, 0, q.n, float(m.config.radius), dev)
    with torch.no_grad():
        ref_f = m.geometry.forward_level(pts)
        ref_p = plain.geometry.forward_level(pts)
    assert torch.equal(q.sdf, ref_f)
    np.testing.assert_allclose(q.sdf.cpu().numpy(), ref_p.cpu().numpy(), rtol=1e-4, atol=3e-5)
    # lattice corners are the box corners
    assert torch.allclose(pts[0], torch.full((3,), -1.0, device=dev))
    assert torch.allclose(pts[-1], torch.full((3,), 1.0, device=dev))
