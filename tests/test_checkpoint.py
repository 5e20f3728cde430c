"""Reference checkpoint interop (angelo_gb.checkpoint): a NeuSModel exported
in the reference's Lightning form (keys under ``model.``, nerfacc 0.3.3
occupancy buffers) loads back bit for bit, strictly, from a dict or a file;
the occupancy mask maps cell c = x res^2 + y res + z to bit c % 32 of word
c / 32 both ways."""
import torch

from angelo_gb import checkpoint, models, workloads


def _model(seed, bg=False):
    torch.manual_seed(seed)
    extra = workloads.background() if bg else {}
    m = models.make("neus", workloads.model_config("small", grid_prune=True, **extra))
    with torch.no_grad():
        for p in m.parameters():
            p.copy_(torch.randn_like(p))
        for g in [m.occupancy_grid] + ([m.occupancy_grid_bg] if bg else []):
            g.occs.copy_(torch.rand_like(g.occs))
            g.bits.copy_(torch.randint(-2 ** 31, 2 ** 31 - 1, g.bits.shape, dtype=torch.int32))
    return m


def _assert_same(a, b):
    sa, sb = a.state_dict(), b.state_dict()
    assert sa.keys() == sb.keys()
    for k in sa:
        assert torch.equal(sa[k], sb[k]), k


def test_reference_form_keys():
    m = _model(0)
    ref = checkpoint.to_reference(m)
    res = m.occupancy_grid.res
    assert ref["model.geometry.encoding.encoding.encoding.params"].dim() == 1
    assert "model.geometry.network.layers.0.weight_g" in ref
    assert "model.geometry.network.layers.0.weight_v" in ref
    assert "model.texture.network.layers.0.weight" in ref
    assert "model.variance.variance" in ref and "model.scene_aabb" in ref
    assert ref["model.occupancy_grid._binary"].shape == (res, res, res)
    assert ref["model.occupancy_grid._binary"].dtype == torch.bool
    assert ref["model.occupancy_grid.resolution"].tolist() == [res] * 3
    assert ref["model.occupancy_grid.grid_coords"].shape == (res ** 3, 3)
    assert not any(k.endswith(".bits") for k in ref)


def test_round_trip_dict_and_file(tmp_path):
    for bg in (False, True):
        m = _model(1, bg)
        ref = checkpoint.to_reference(m)
        m2 = _model(2, bg)
        checkpoint.load_reference_checkpoint(m2, {"state_dict": ref, "epoch": 3, "global_step": 7})
        _assert_same(m, m2)
        path = tmp_path / f"ref{int(bg)}.ckpt"
        torch.save({"state_dict": ref}, path)
        m3 = _model(3, bg)
        checkpoint.load_reference_checkpoint(m3, str(path))
        _assert_same(m, m3)


def test_binary_cell_order():
    m = _model(4)
    res = m.occupancy_grid.res
    ref = checkpoint.to_reference(m)
    b = torch.zeros(res, res, res, dtype=torch.bool)
    b[1, 2, 3] = True
    b[res - 1, res - 1, res - 1] = True
    ref["model.occupancy_grid._binary"] = b
    checkpoint.load_reference_checkpoint(m, ref)
    c0 = 1 * res * res + 2 * res + 3
    bits = m.occupancy_grid.bits
    assert int(bits[c0 // 32]) == 1 << (c0 % 32)
    assert int(bits.ne(0).sum()) == 2
    assert torch.equal(m.occupancy_grid.binary, b)


class _Hyper:
    """Stands for the pickled hyper-parameter object of a Lightning checkpoint."""

    def __init__(self):
        self.lr = 0.01


def test_pickled_objects_need_trusted(tmp_path):
    """A checkpoint that pickles an object is refused unless trusted=True."""
    import pytest
    m = _model(5)
    ref = checkpoint.to_reference(m)
    path = tmp_path / "with_object.ckpt"
    torch.save({"state_dict": ref, "hyper_parameters": _Hyper()}, path)
    m2 = _model(6)
    with pytest.raises(RuntimeError, match="trusted=True"):
        checkpoint.load_reference_checkpoint(m2, str(path))
    checkpoint.load_reference_checkpoint(m2, str(path), trusted=True)
    _assert_same(m, m2)


def test_pack_unpack_bits_round_trip():
    """pack_bits / unpack_bits: bit c % 32 of word c // 32, sizes that are not
    multiples of 32, the sign bit included."""
    g = torch.Generator().manual_seed(9)
    for n in (1, 31, 32, 33, 1000, 4097):
        m = torch.rand(n, generator=g) < 0.5
        w = checkpoint.pack_bits(m)
        assert w.dtype == torch.int32 and w.numel() == (n + 31) // 32
        assert torch.equal(checkpoint.unpack_bits(w, n), m)
        for c in torch.nonzero(m)[:, 0].tolist()[:20]:
            assert (int(w[c // 32]) >> (c % 32)) & 1 == 1
    full = torch.ones(64, dtype=torch.bool)
    assert checkpoint.pack_bits(full).tolist() == [-1, -1]
