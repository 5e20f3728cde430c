"""The library seam (angelo_gb.seam): the tinycudann / nerfacc 0.3.3
stand-ins the reference's model code imports, on libangelo_gb.so, against
the oracle's restatements of those packages (oracle/cref.py, the same
restatements the golden vectors of the reference's own model code were made
with) and against the drop-in model on the same inputs:

* tcnn.Encoding(HashGrid): float32 encoding bit-exact with the C oracle,
  table gradient against a float64 scatter of the oracle's corner weights;
  SphericalHarmonics against the oracle's basis;
* nerfacc.ray_marching through an OccupancyGrid: ray indices and t bit-exact
  with the C oracle (plain and with the sigma_fn visibility test);
* render_weight_from_alpha bit-exact with the C oracle's weights;
  accumulate_along_rays and render_weight_from_density against float64;
* a NeuS forward written the way models/neus.py:205-283 calls the two
  packages, on the drop-in geometry and texture modules, equal to the
  drop-in NeuSModel.forward_ (plain form) on the same rays."""
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


@pytest.fixture(scope="module")
def seam():
    from angelo_gb import seam as S
    return S.modules()


HG = dict(otype="HashGrid", n_levels=16, n_features_per_level=2, log2_hashmap_size=19,
          base_resolution=32, per_level_scale=1.3195079107728942)


def test_encoding_hashgrid_matches_oracle(dev, seam):
    from oracle import cref
    from oracle import neus_fp64 as O
    tcnn = seam["tinycudann"]
    enc = tcnn.Encoding(3, HG).to(dev)
    assert enc.n_output_dims == 32 and enc.n_input_dims == 3
    with torch.no_grad():
        g = torch.Generator(device="cpu").manual_seed(1)
        enc.params.copy_((torch.rand(enc.params.shape, generator=g) * 0.1 - 0.05).to(dev))
    x = torch.rand(4096, 3, generator=torch.Generator(device="cpu").manual_seed(2))
    x[:8] = torch.tensor([0.0, 1.0, 0.5])          # edges of the unit cube
    xd = x.to(dev).requires_grad_(False)
    out = enc(xd)
    lay = O.HashGridLayout(16, 2, 19, 32, HG["per_level_scale"])
    ref = cref.hashgrid_encode(x.numpy(), enc.params.detach().cpu().numpy(), lay.cref_layout)
    assert np.array_equal(out.detach().cpu().numpy(), ref)
    # table gradient of a weighted sum: the float64 scatter of the C oracle's
    # float32 corner weights (tcnn's position arithmetic is float32, so its
    # weights differ from exact ones by ~ulp(scale * x) at the fine levels)
    wsum = torch.randn(4096, 32, generator=torch.Generator(device="cpu").manual_seed(3))
    (out * wsum.to(dev)).sum().backward()
    idx, w = cref.hashgrid_index(x.numpy(), lay.cref_layout)
    ent = idx.astype(np.int64) + np.asarray(lay.offsets[:16], np.int64)[None, :, None]
    g = wsum.double().numpy().reshape(4096, 16, 1, 2) * w.astype(np.float64)[..., None]
    ref_g = np.zeros((lay.n_entries, 2))
    np.add.at(ref_g, ent.reshape(-1), g.reshape(-1, 2))
    got = enc.params.grad.cpu().double().numpy().reshape(-1, 2)
    # float32 atomics of terms up to |wsum|: accumulation order only
    np.testing.assert_allclose(got, ref_g, rtol=1e-5, atol=2e-6)


def test_encoding_sh_matches_oracle(dev, seam):
    from oracle import neus_fp64 as O
    enc = seam["tinycudann"].Encoding(3, dict(otype="SphericalHarmonics", degree=4))
    d = torch.nn.functional.normalize(torch.randn(1000, 3, generator=torch.Generator().manual_seed(4)),
                                      dim=-1)
    d01 = (d + 1) / 2
    out = enc(d01.to(dev))
    np.testing.assert_allclose(out.cpu().double().numpy(), O.sh4(d01.double()).numpy(), atol=2e-6)


def test_unprovided_tcnn_entry_points_raise(seam):
    tcnn = seam["tinycudann"]
    with pytest.raises(NotImplementedError):
        tcnn.Network(3, 1, {"otype": "FullyFusedMLP"})
    with pytest.raises(NotImplementedError):
        tcnn.Encoding(3, {"otype": "Frequency", "n_frequencies": 4})


def _rays(dev, n=512, seed=5, radius=0.5):
    g = np.random.default_rng(seed)
    eye = g.normal(size=(n, 3))
    eye = 1.5 * eye / np.linalg.norm(eye, axis=1, keepdims=True)
    tgt = g.uniform(-0.3 * radius, 0.3 * radius, (n, 3))
    d = tgt - eye
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return torch.tensor(np.concatenate([eye, d], 1), dtype=torch.float32, device=dev)


def _grid(seam, dev, res=32, seed=6):
    nerfacc = seam["nerfacc"]
    aabb = torch.tensor([-0.5, -0.5, -0.5, 0.5, 0.5, 0.5])
    grid = nerfacc.OccupancyGrid(roi_aabb=aabb, resolution=res,
                                 contraction_type=nerfacc.ContractionType.AABB).to(dev)
    occ = torch.rand(res ** 3, generator=torch.Generator().manual_seed(seed)) < 0.3
    from angelo_gb.checkpoint import pack_bits
    grid.bits.copy_(pack_bits(occ).to(dev))
    return grid, aabb, occ.reshape(res, res, res)


def test_ray_marching_matches_oracle(dev, seam):
    from oracle import cref
    nerfacc = seam["nerfacc"]
    grid, aabb, occ = _grid(seam, dev)
    rays = _rays(dev)
    o, d = rays[:, :3], rays[:, 3:]
    step = 1.732 * 2 * 0.5 / 256
    ri, t0, t1 = nerfacc.ray_marching(o, d, scene_aabb=aabb.to(dev), grid=grid,
                                      render_step_size=step, stratified=False, cone_angle=0.0,
                                      alpha_thre=0.0)
    assert ri.dtype == torch.int32 and t0.shape == (ri.numel(), 1)
    tmin, tmax = cref.ray_aabb(o.cpu().numpy(), d.cpu().numpy(), aabb.numpy())
    _, off, r_ri, r_t0, r_t1, _ = cref.march(o.cpu().numpy(), d.cpu().numpy(), tmin, tmax,
                                             aabb.numpy(), occ.numpy().astype(np.uint8), step)
    assert ri.numel() > 1000
    assert np.array_equal(ri.cpu().numpy(), r_ri)
    assert np.array_equal(t0.view(-1).cpu().numpy(), r_t0)
    assert np.array_equal(t1.view(-1).cpu().numpy(), r_t1)
    ti, ta = seam["nerfacc.intersection"].ray_aabb_intersect(o, d, aabb.to(dev))
    assert np.array_equal(ti.cpu().numpy(), tmin) and np.array_equal(ta.cpu().numpy(), tmax)


def test_ray_marching_visibility_test(dev, seam):
    """sigma_fn: samples behind transmittance < early_stop_eps are dropped
    (nerfacc 0.3.3's render_visibility), computed here in float64 from the
    same samples."""
    from oracle import cref
    nerfacc = seam["nerfacc"]
    grid, aabb, _ = _grid(seam, dev, seed=7)
    rays = _rays(dev, 256, seed=8)
    o, d = rays[:, :3], rays[:, 3:]
    step = 1.732 * 2 * 0.5 / 256

    def sigma_fn(ts, te, ri):
        p = o[ri] + d[ri] * (ts + te) / 2
        return 400.0 * torch.exp(-(p.norm(dim=-1, keepdim=True) / 0.25) ** 2)

    all_ri, all_t0, all_t1 = nerfacc.ray_marching(o, d, scene_aabb=aabb.to(dev), grid=grid,
                                                  render_step_size=step)
    ri, t0, t1 = nerfacc.ray_marching(o, d, scene_aabb=aabb.to(dev), grid=grid, sigma_fn=sigma_fn,
                                      render_step_size=step)
    assert 0 < ri.numel() < all_ri.numel()
    sig = sigma_fn(all_t0, all_t1, all_ri.long()).view(-1).double()
    alpha = 1 - torch.exp(-sig * (all_t1 - all_t0).view(-1).double())
    off = torch.cat([torch.zeros(1, dtype=torch.int64),
                     torch.cumsum(torch.bincount(all_ri.long().cpu(), minlength=256), 0)]).numpy()
    _, trans = cref.weights(alpha.float().cpu().numpy(), off)
    keep = torch.from_numpy(trans >= 1e-4).to(dev)
    assert torch.equal(ri, all_ri[keep]) and torch.equal(t0, all_t0[keep])


def test_weights_and_accumulate(dev, seam):
    from oracle import cref
    nerfacc = seam["nerfacc"]
    g = torch.Generator().manual_seed(9)
    counts = torch.randint(0, 60, (300,), generator=g)
    ri = torch.repeat_interleave(torch.arange(300), counts).int().to(dev)
    n = ri.numel()
    alpha = (torch.rand(n, 1, generator=g) ** 3).to(dev)
    w = nerfacc.render_weight_from_alpha(alpha, ray_indices=ri, n_rays=300)
    off = np.concatenate([[0], np.cumsum(counts.numpy())]).astype(np.int64)
    rw, _ = cref.weights(alpha.view(-1).cpu().numpy(), off)
    assert w.shape == alpha.shape and np.array_equal(w.view(-1).cpu().numpy(), rw)
    vals = torch.randn(n, 3, generator=g).to(dev)
    acc = nerfacc.accumulate_along_rays(w, ri, values=vals, n_rays=300)
    ref = torch.zeros(300, 3, dtype=torch.float64, device=dev).index_add(
        0, ri.long(), w.double() * vals.double())
    assert acc.shape == (300, 3)
    torch.testing.assert_close(acc.double(), ref, rtol=1e-5, atol=1e-6)
    op = nerfacc.accumulate_along_rays(w, ri, values=None, n_rays=300)
    assert op.shape == (300, 1)
    t0 = torch.rand(n, 1, generator=g).to(dev)
    t1 = t0 + 0.01
    sig = (torch.rand(n, 1, generator=g) * 50).to(dev)
    wd = nerfacc.render_weight_from_density(t0, t1, sig, ray_indices=ri, n_rays=300)
    tau = (sig * (t1 - t0)).double().view(-1)
    ref_w = []
    for r in range(300):
        s = tau[off[r]:off[r + 1]]
        ex = torch.cat([torch.zeros(1, dtype=s.dtype, device=dev), torch.cumsum(s, 0)[:-1]])
        ref_w.append((1 - torch.exp(-s)) * torch.exp(-ex))
    torch.testing.assert_close(wd.view(-1).double(), torch.cat(ref_w), rtol=1e-5, atol=1e-6)


def test_neus_forward_on_the_seam_equals_dropin(dev, seam):
    """NeuSModel.forward_'s calls of the two packages (models/neus.py:
    205-283), written against the seam's tinycudann / nerfacc, on the drop-in
    geometry and texture modules: the same per-ray outputs as the drop-in
    model's own forward (plain form, identical samples)."""
    import torch.nn.functional as F
    from angelo_gb import models, workloads
    nerfacc = seam["nerfacc"]
    torch.manual_seed(0)
    m = models.make("neus", workloads.model_config("full")).to(dev)
    m.update_step(0, 6000)
    m.train()
    m.randomized = False
    with torch.no_grad():
        p = m.geometry.hashgrid.encoding.params
        p.copy_((torch.rand(p.shape, generator=torch.Generator().manual_seed(1)) * 0.1 - 0.05).to(dev))
    from angelo_gb import scenes
    occ = scenes.analytic_occupancy(scenes.UnionScene(), 128, device=dev).reshape(-1)
    from angelo_gb.checkpoint import pack_bits
    m.occupancy_grid.bits.copy_(pack_bits(occ.cpu()).to(dev))
    grid = nerfacc.OccupancyGrid(roi_aabb=m.scene_aabb, resolution=128,
                                 contraction_type=nerfacc.ContractionType.AABB).to(dev)
    grid.bits.copy_(m.occupancy_grid.bits)
    rays = _rays(dev, 256, seed=10)
    S_ = 0
    ri0, _, _, _ = m.march_rays(rays[:, :3].contiguous(), rays[:, 3:].contiguous())
    S_ = ri0.numel()
    rd = torch.randn(S_, 3, generator=torch.Generator().manual_seed(11)).to(dev)
    m.geometry.curvature_dirs_fn = lambda t: rd
    bg = torch.tensor([0.2, 0.4, 0.6], device=dev)
    m.background_color = bg
    with torch.no_grad():
        ref = m.forward_(rays)

        n_rays = rays.shape[0]
        rays_o, rays_d = rays[:, 0:3], rays[:, 3:6]
        ray_indices, t_starts, t_ends = nerfacc.ray_marching(
            rays_o, rays_d, scene_aabb=m.scene_aabb, grid=grid, alpha_fn=None, near_plane=None,
            far_plane=None, render_step_size=m.render_step_size, stratified=False, cone_angle=0.0,
            alpha_thre=0.0)
        ray_indices = ray_indices.long()
        t_origins, t_dirs = rays_o[ray_indices], rays_d[ray_indices]
        midpoints = (t_starts + t_ends) / 2.0
        positions = t_origins + t_dirs * midpoints
        dists = t_ends - t_starts
        sdf, sdf_grad, feature, sdf_laplace = m.geometry(positions, with_grad=True, with_feature=True,
                                                          with_laplace=True)
        normal = F.normalize(sdf_grad, p=2, dim=-1)
        alpha = m.get_alpha(sdf, normal, t_dirs, dists)[..., None]
        rgb = m.texture(feature, t_dirs, normal)
        weights = nerfacc.render_weight_from_alpha(alpha, ray_indices=ray_indices, n_rays=n_rays)
        opacity = nerfacc.accumulate_along_rays(weights, ray_indices, values=None, n_rays=n_rays)
        depth = nerfacc.accumulate_along_rays(weights, ray_indices, values=midpoints, n_rays=n_rays)
        comp_rgb = nerfacc.accumulate_along_rays(weights, ray_indices, values=rgb, n_rays=n_rays)
        comp_rgb_full = comp_rgb + bg * (1.0 - opacity)
    assert ray_indices.numel() == S_
    for a, b in ((opacity, ref["opacity"]), (depth, ref["depth"]), (comp_rgb_full, ref["comp_rgb_full"]),
                 (weights.view(-1), ref["weights"].view(-1))):
        torch.testing.assert_close(a, b.reshape(a.shape), rtol=0, atol=1e-6)
