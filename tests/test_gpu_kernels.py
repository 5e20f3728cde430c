"""Kernel parity on the GPU, through the C ABI: integer outputs bit-exact
against the C oracle; float32 outputs that the oracle computes in the same
float32 order also bit-exact; everything else against the FP64 oracle within
the tolerance written in each test."""
import numpy as np
import pytest
import torch

from oracle import cref
from oracle import neus_fp64 as O

pytestmark = pytest.mark.gpu

CONFIGS = {
    "c1": (8, 16, 16, 1.5),
    "c2": (16, 22, 32, 1.3195079107728942),
    "small": (16, 10, 4, 1.3195079107728942),
}


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from angelo_gb import build
    build.build()
    return torch.device("cuda:0")


def _points(n, seed, with_edges=True):
    g = np.random.default_rng(seed)
    x = g.random((n, 3), dtype=np.float32)
    if with_edges:
        x[:8] = np.array([[0, 0, 0], [1, 1, 1], [0, 1, 0], [1, 0, 1], [0.5, 0.5, 0.5],
                          [1e-7, 1 - 1e-7, 0.25], [0.999999, 0.0000001, 0.75],
                          [1.0 / 3, 2.0 / 3, 0.1]], np.float32)
    return x


@pytest.mark.parametrize("cfg", list(CONFIGS))
def test_hash_indices_bit_exact(dev, cfg):
    from angelo_gb.ops import HashGridSpec, hashgrid_index
    L, log2T, base, b = CONFIGS[cfg]
    spec = HashGridSpec(L, 2, log2T, base, b)
    x = _points(20000, 1)
    # points slightly outside [0,1] (clamped FD stencils never produce them,
    # but the reference encodes whatever it is given)
    x[8:16] = np.array([[-0.01, 0.5, 0.5], [1.02, 0.3, 0.2], [0.5, -0.2, 1.1]] * 2 +
                       [[-1, -1, -1], [2, 2, 2]], np.float32)
    idx, w = hashgrid_index(torch.from_numpy(x).to(dev), spec)
    ridx, rw = cref.hashgrid_index(x, cref.hashgrid_layout(L, log2T, base, b))
    np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32), ridx)
    np.testing.assert_array_equal(w.cpu().numpy(), rw)


@pytest.mark.parametrize("cfg", list(CONFIGS))
def test_encode_fp32_bit_exact(dev, cfg):
    from angelo_gb.ops import HashGridSpec, hashgrid_encode_raw
    L, log2T, base, b = CONFIGS[cfg]
    spec = HashGridSpec(L, 2, log2T, base, b)
    rng = np.random.default_rng(2)
    table = rng.uniform(-1, 1, spec.n_params).astype(np.float32)
    x = _points(30000, 3)
    t = torch.from_numpy(table).to(dev)
    xt = torch.from_numpy(x).to(dev)
    lay = cref.hashgrid_layout(L, log2T, base, b)
    for active in (L, 4, 0):
        out = hashgrid_encode_raw(xt, t, spec, active, include_xyz=True).cpu().numpy()
        ref = cref.hashgrid_encode(x, table, lay, active_levels=active)
        np.testing.assert_array_equal(out[:, 3:], ref)
        np.testing.assert_array_equal(out[:, :3], x * 2 - 1)


def test_encode_fp16_table(dev):
    from angelo_gb.ops import HashGridSpec, hashgrid_encode_raw
    L, log2T, base, b = CONFIGS["c1"]
    spec = HashGridSpec(L, 2, log2T, base, b)
    rng = np.random.default_rng(4)
    table = rng.uniform(-1, 1, spec.n_params).astype(np.float16)
    x = _points(10000, 5)
    out = hashgrid_encode_raw(torch.from_numpy(x).to(dev), torch.from_numpy(table).to(dev), spec,
                              L, include_xyz=False).cpu().numpy()
    ref = cref.hashgrid_encode(x, table.astype(np.float32), cref.hashgrid_layout(L, log2T, base, b))
    # fp16 storage, fp32 interpolation: only the accumulation order differs
    np.testing.assert_allclose(out, ref, rtol=1e-6, atol=1e-6)


def test_encode_backward_against_fp64(dev):
    from angelo_gb.ops import HashGridSpec, hashgrid_encode
    L, log2T, base, b = CONFIGS["small"]
    spec = HashGridSpec(L, 2, log2T, base, b)
    lay = O.HashGridLayout(L, 2, log2T, base, b)
    rng = np.random.default_rng(6)
    table = rng.uniform(-1, 1, spec.n_params).astype(np.float32)
    x = rng.uniform(0.02, 0.98, (3000, 3)).astype(np.float32)
    gout = rng.normal(size=(3000, 3 + 2 * L)).astype(np.float32)
    for active in (L, 5):
        xt = torch.from_numpy(x).to(dev).requires_grad_(True)
        tt = torch.from_numpy(table).to(dev).requires_grad_(True)
        out = hashgrid_encode(xt, tt, spec, active, include_xyz=True)
        (out * torch.from_numpy(gout).to(dev)).sum().backward()
        x64 = torch.tensor(x, dtype=torch.float64, requires_grad=True)
        t64 = torch.tensor(table, dtype=torch.float64, requires_grad=True)
        o64 = O.composite_encode(x64, t64, lay, active)
        (o64 * torch.tensor(gout, dtype=torch.float64)).sum().backward()
        # table gradient: float32 atomics of w*g, order not fixed
        np.testing.assert_allclose(tt.grad.cpu().numpy(), t64.grad.numpy(), rtol=1e-4, atol=1e-4)
        # input gradient: sums over levels of scale * table differences, with
        # cancellation; compared relative to the largest component
        ref = x64.grad.numpy()
        np.testing.assert_allclose(xt.grad.cpu().numpy(), ref, rtol=1e-4,
                                   atol=2e-5 * np.abs(ref).max())


def test_sh4(dev):
    from angelo_gb.ops import sh4_encode
    rng = np.random.default_rng(7)
    d = rng.normal(size=(5000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    d01 = ((d + 1) / 2).astype(np.float32)
    out = sh4_encode(torch.from_numpy(d01).to(dev)).cpu().numpy()
    np.testing.assert_allclose(out, cref.sh4(d01), rtol=1e-5, atol=2e-6)
    # backward against FP64 autograd
    dt = torch.from_numpy(d01).to(dev).requires_grad_(True)
    g = rng.normal(size=(5000, 16)).astype(np.float32)
    (sh4_encode(dt) * torch.from_numpy(g).to(dev)).sum().backward()
    d64 = torch.tensor(d01, dtype=torch.float64, requires_grad=True)
    (O.sh4(d64) * torch.tensor(g, dtype=torch.float64)).sum().backward()
    np.testing.assert_allclose(dt.grad.cpu().numpy(), d64.grad.numpy(), rtol=1e-4, atol=1e-4)


def _rays(n, seed, radius=0.5):
    g = np.random.default_rng(seed)
    o = g.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 2.5 * radius * 2
    d = -o / np.linalg.norm(o, axis=1, keepdims=True) + g.uniform(-0.3, 0.3, (n, 3))
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def _random_bits(res, p, seed):
    g = np.random.default_rng(seed)
    b = (g.random(res ** 3) < p).astype(np.uint8)
    words = np.packbits(b, bitorder="little").view(np.uint32) if res ** 3 >= 32 else None
    return b.reshape(res, res, res), words


@pytest.mark.parametrize("p_occ,r,res", [(1.0, 0.5, 128), (0.3, 0.5, 128), (0.02, 0.5, 128),
                                         (0.0, 0.5, 128), (0.3, 0.7, 96), (0.02, 0.7, 96)])
def test_march_bit_exact(dev, p_occ, r, res):
    """Power-of-two extents and resolutions (0.5 box, 128^3) take the kernel's
    exact multiplication form of the divisions; 1.4 and 96 keep the divisions."""
    from angelo_gb import ops
    o, d = _rays(4096, 8, r)
    o[0] = [3, 3, 3]  # misses the box
    d[0] = [1, 0, 0]
    aabb = np.array([-r, -r, -r, r, r, r], np.float32)
    tmin, tmax = ops.ray_aabb_intersect(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                        torch.from_numpy(aabb).to(dev))
    rtmin, rtmax = cref.ray_aabb(o, d, aabb)
    np.testing.assert_array_equal(tmin.cpu().numpy(), rtmin)
    np.testing.assert_array_equal(tmax.cpu().numpy(), rtmax)
    jit = np.random.default_rng(9).random(4096, dtype=np.float32)
    step = 1.732 * 2 * r / 1024
    tmin_j = (rtmin + jit * np.float32(step)).astype(np.float32)
    binary, words = _random_bits(res, p_occ, 10)
    ri, t0, t1, off, st = ops.march(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                    torch.from_numpy(tmin_j).to(dev), tmax, step, roi=aabb,
                                    res=(res, res, res),
                                    bits=torch.from_numpy(words.view(np.int32)).to(dev))
    cnt, roff, rri, rt0, rt1, ovf = cref.march(o, d, tmin_j, rtmax, aabb, binary, step)
    np.testing.assert_array_equal(off.cpu().numpy(), roff)
    np.testing.assert_array_equal(ri.cpu().numpy(), rri)
    np.testing.assert_array_equal(t0.cpu().numpy(), rt0)
    np.testing.assert_array_equal(t1.cpu().numpy(), rt1)
    assert int(st) == 0 and not ovf
    if p_occ == 0.0:
        assert off[-1].item() == 0


@pytest.mark.parametrize("per_ray", [None, 1026, 7])
def test_march_single_pass_matches_oracle(dev, per_ray):
    """The single-march path (samples recorded while counting, compacted after
    the scan) against the oracle; per_ray 7 overflows and falls back to the
    second march, with the same samples."""
    from angelo_gb import ops
    r = 1.0
    o, d = _rays(2048, 21, 2.0)
    aabb = np.array([-r, -r, -r, r, r, r], np.float32)
    tmin, tmax = ops.ray_aabb_intersect(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                        torch.from_numpy(aabb).to(dev))
    rtmin, rtmax = cref.ray_aabb(o, d, aabb)
    jit = np.random.default_rng(22).random(2048, dtype=np.float32)
    step = 1.732 * 2 * r / 1024
    tmin_j = (rtmin + jit * np.float32(step)).astype(np.float32)
    binary, words = _random_bits(128, 0.3, 23)
    ri, t0, t1, off, st = ops.march(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                    torch.from_numpy(tmin_j).to(dev), tmax, step, roi=aabb,
                                    res=(128, 128, 128),
                                    bits=torch.from_numpy(words.view(np.int32)).to(dev),
                                    max_samples_per_ray=per_ray)
    _, roff, rri, rt0, rt1, _ = cref.march(o, d, tmin_j, rtmax, aabb, binary, step)
    np.testing.assert_array_equal(off.cpu().numpy(), roff)
    np.testing.assert_array_equal(ri.cpu().numpy(), rri)
    np.testing.assert_array_equal(t0.cpu().numpy(), rt0)
    np.testing.assert_array_equal(t1.cpu().numpy(), rt1)
    assert (int(st) & 3) == 0
    if per_ray == 7:
        assert int(st) & 4   # the bound was exceeded: second march used


@pytest.mark.parametrize("per_ray", [None, 1200, 7])
def test_march_count_read_through_event_matches(dev, per_ray):
    """The training step's count read (a pinned copy and an event, with the
    caller's work enqueued between them) gives the same samples, flags and
    offsets as the plain read, and the caller's work runs before the outputs
    are sized."""
    from angelo_gb import ops
    r = 1.0
    o, d = _rays(2048, 24, 2.0)
    aabb = np.array([-r, -r, -r, r, r, r], np.float32)
    ot, dt = torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev)
    tmin, tmax = ops.ray_aabb_intersect(ot, dt, torch.from_numpy(aabb).to(dev))
    binary, words = _random_bits(128, 0.3, 25)
    grid = dict(roi=aabb, res=(128, 128, 128), bits=torch.from_numpy(words.view(np.int32)).to(dev),
                max_samples_per_ray=per_ray)
    step = 1.732 * 2 * r / 1024
    ref = ops.march(ot, dt, tmin, tmax, step, **grid)
    side = torch.zeros(1 << 20, device=dev)
    calls = []

    def before_read():
        calls.append(1)
        side.add_(1.0)   # work on the stream between the copy and the wait

    got = ops.march(ot, dt, tmin, tmax, step, before_read=before_read, **grid)
    assert calls == [1] and float(side[-1]) == 1.0
    for a, b in zip(ref[:4], got[:4]):
        assert torch.equal(a, b)
    assert int(ref[4]) == int(got[4])


def test_march_without_grid_between_planes(dev):
    """Config-1 style: no grid, samples between near 0.5 and far 4.5, dt 1/32."""
    from angelo_gb import ops
    o, d = _rays(1024, 11, 1.0)
    n = len(o)
    tmin = np.full(n, 0.5, np.float32)
    tmax = np.full(n, 4.5, np.float32)
    ri, t0, t1, off, _ = ops.march(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                   torch.from_numpy(tmin).to(dev), torch.from_numpy(tmax).to(dev),
                                   1.0 / 32)
    assert np.all(np.diff(off.cpu().numpy()) == 128)
    _, roff, rri, rt0, rt1, _ = cref.march(o, d, tmin, tmax, np.array([-1e10] * 3 + [1e10] * 3,
                                                                      np.float32),
                                           np.ones((1, 1, 1), np.uint8), 1.0 / 32)
    np.testing.assert_array_equal(t0.cpu().numpy(), rt0)


def test_march_step_cap_sets_status(dev):
    from angelo_gb import ops
    o = np.zeros((2, 3), np.float32)
    d = np.array([[1, 0, 0], [0, 1, 0]], np.float32)
    ri, t0, t1, off, st = ops.march(torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev),
                                    torch.zeros(2, device=dev), torch.full((2,), 1e10, device=dev),
                                    0.01, max_steps=1000)
    assert int(st) & 1
    assert np.all(np.diff(off.cpu().numpy()) == 1000)


@pytest.mark.parametrize("n", [0, 1, 1023, 1024, 1025, 300000, 4 * 1024 * 1024 + 7])
def test_scan(dev, n):
    from angelo_gb import ops
    c = np.random.default_rng(n).integers(0, 700, n).astype(np.int32)
    off = ops.scan(torch.from_numpy(c).to(dev)).cpu().numpy()
    ref = np.zeros(n + 1, np.int64)
    np.cumsum(c, out=ref[1:])
    np.testing.assert_array_equal(off, ref)


def test_weights_and_accumulate(dev):
    from angelo_gb import ops
    rng = np.random.default_rng(12)
    counts = rng.integers(0, 300, 500)
    counts[:3] = [0, 1, 2000]
    off = np.zeros(len(counts) + 1, np.int64)
    np.cumsum(counts, out=off[1:])
    S = int(off[-1])
    alpha = rng.random(S, dtype=np.float32) ** 4
    alpha[off[5]:off[6]] = 1.0  # an opaque ray
    offt = torch.from_numpy(off).to(dev)
    at = torch.from_numpy(alpha).to(dev).requires_grad_(True)
    w = ops.render_weight_from_alpha(at, offt)
    rw, _ = cref.weights(alpha, off)
    np.testing.assert_array_equal(w.detach().cpu().numpy(), rw)   # same float32 sequence
    vals = rng.normal(size=(S, 3)).astype(np.float32)
    vt = torch.from_numpy(vals).to(dev).requires_grad_(True)
    acc = ops.accumulate_along_rays(w[:, None], offt, vt)
    opa = ops.accumulate_along_rays(w[:, None], offt)
    g1 = rng.normal(size=(len(counts), 3)).astype(np.float32)
    g2 = rng.normal(size=(len(counts), 1)).astype(np.float32)
    ((acc * torch.from_numpy(g1).to(dev)).sum() + (opa * torch.from_numpy(g2).to(dev)).sum()).backward()
    a64 = torch.tensor(alpha, dtype=torch.float64, requires_grad=True)
    v64 = torch.tensor(vals, dtype=torch.float64, requires_grad=True)
    w64 = O.render_weights(a64, list(off))
    ri = torch.repeat_interleave(torch.arange(len(counts)), torch.from_numpy(counts))
    acc64 = O.accumulate(w64, ri, v64, len(counts))
    opa64 = O.accumulate(w64, ri, None, len(counts))
    ((acc64 * torch.tensor(g1, dtype=torch.float64)).sum() +
     (opa64 * torch.tensor(g2, dtype=torch.float64)).sum()).backward()
    np.testing.assert_allclose(acc.detach().cpu().numpy(), acc64.detach().numpy(), rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(opa.detach().cpu().numpy(), opa64.detach().numpy(), rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(at.grad.cpu().numpy(), a64.grad.numpy(), rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(vt.grad.cpu().numpy(), v64.grad.numpy(), rtol=1e-5, atol=1e-6)


def test_occupancy_update(dev):
    from angelo_gb import ops
    rng = np.random.default_rng(13)
    n_cells = 128 ** 3
    occs = (rng.random(n_cells, dtype=np.float32) * 0.01).astype(np.float32)
    # warm-up style: every cell once
    cells = np.arange(n_cells, dtype=np.int64)
    occ = (rng.random(n_cells, dtype=np.float32) ** 8).astype(np.float32)
    o_t = torch.from_numpy(occs).to(dev)
    bits = torch.zeros(n_cells // 32, dtype=torch.int32, device=dev)
    ops.occ_update(o_t, torch.from_numpy(cells).to(dev), torch.from_numpy(occ).to(dev), 0.95,
                   0.001, bits)
    ref = np.maximum(occs * np.float32(0.95), occ)
    np.testing.assert_array_equal(o_t.cpu().numpy(), ref)
    np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint32), cref.occ_binary(ref, 0.001))
    # sampled cells with duplicates: scatter-max per cell, decay once
    k = n_cells // 4
    cells2 = rng.integers(0, n_cells, k).astype(np.int64)
    occ2 = rng.random(k, dtype=np.float32)
    before = o_t.cpu().numpy().copy()
    ops.occ_update(o_t, torch.from_numpy(cells2).to(dev), torch.from_numpy(occ2).to(dev), 0.95,
                   0.001, bits)
    ref2 = before.copy()
    mx = np.full(n_cells, -1.0, np.float32)
    np.maximum.at(mx, cells2, occ2)
    touched = mx >= 0
    ref2[touched] = np.maximum(before[touched] * np.float32(0.95), mx[touched])
    np.testing.assert_array_equal(o_t.cpu().numpy(), ref2)
    np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint32), cref.occ_binary(ref2, 0.001))
