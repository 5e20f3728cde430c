"""Host-side checks that need no GPU: the C-ABI library loads and exports
every symbol its header declares, the host-only layout call matches the
oracle bit for bit, and the drop-in modules build with the reference's
configuration keys and parameter names."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import cref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    txt = open(os.path.join(ROOT, "include", "angelo_gb.h")).read()
    return sorted(set(re.findall(r"\b(angelo_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from angelo_gb import build, _lib
    build.build()
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    syms = _declared_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(lib, s), s
    from angelo_gb import _lib
    assert set(_lib.SIGNATURES) == set(syms)


@pytest.mark.parametrize("cfg", [(8, 16, 16, 1.5), (16, 22, 32, 1.3195079107728942),
                                 (16, 19, 32, 1.3195079107728942), (16, 10, 4, 1.3195079107728942)])
def test_layout_matches_oracle(lib, cfg):
    from angelo_gb.ops import HashGridSpec
    L, log2T, base, b = cfg
    spec = HashGridSpec(L, 2, log2T, base, b)
    off, res, sc = cref.hashgrid_layout(L, log2T, base, b)
    assert spec.offsets == [int(v) for v in off]
    assert spec.resolutions == [int(v) for v in res]
    assert np.array_equal(np.array(spec.scales, np.float32), sc)


def test_layout_rejects_bad_config(lib):
    from angelo_gb import _lib
    from angelo_gb.ops import HashGridSpec
    with pytest.raises(_lib.AngeloError) as e:
        HashGridSpec(40, 2, 19, 16, 1.5)
    assert e.value.code == _lib.ANGELO_E_INVALID
    with pytest.raises(_lib.AngeloError):
        HashGridSpec(8, 4, 19, 16, 1.5)


def test_workspace_queries(lib):
    assert lib.angelo_scan_workspace_size(0) >= 8
    assert lib.angelo_scan_workspace_size(10 ** 6) >= 8 * (10 ** 6 // 1024)
    assert lib.angelo_occ_workspace_size(128 ** 3) >= 4 * 128 ** 3


def test_dropins_build_with_reference_keys(lib):
    from angelo_gb import models
    from golden_util import load
    g = load("neus_dual_grid")
    from golden_util import model_config
    m = models.make("neus", model_config(g))
    names = set(m.state_dict().keys())
    ref = {k[len("param/"):] for k in g if k.startswith("param/")}
    assert ref <= names, ref - names
    for k in ref:
        assert tuple(m.state_dict()[k].shape) == g["param/" + k].shape, k


def test_ctypes_signatures_match_header_argument_counts(lib):
    """Every declared entry point is bound with as many ctypes arguments as the
    header declares (a mismatch would pass garbage through the C ABI)."""
    from angelo_gb import _lib
    txt = open(os.path.join(ROOT, "include", "angelo_gb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    n_checked = 0
    for m in re.finditer(r"\b(angelo_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt):
        name, args = m.group(1), m.group(2).strip()
        n = 0 if args in ("", "void") else len(args.split(","))
        assert name in _lib.SIGNATURES, name
        assert len(_lib.SIGNATURES[name][1]) == n, (name, n, len(_lib.SIGNATURES[name][1]))
        n_checked += 1
    assert n_checked == len(_lib.SIGNATURES)


def test_unbound_entry_point_is_refused(lib):
    from angelo_gb import _lib
    with pytest.raises(_lib.AngeloError):
        _lib.call("angelo_not_declared", 1, 2)


def test_ide_matches_reference_golden():
    """angelo_gb.ide (Legendre-derivative polynomials) against the reference's
    generate_ide_fn(4) golden vectors."""
    import os
    import torch
    from angelo_gb.ide import IntegratedDirEncoding
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ide_deg4.npz"))
    enc = IntegratedDirEncoding(4).double()
    out = enc(torch.from_numpy(g["xyz"]).double(), torch.from_numpy(g["kappa_inv"]).double())
    assert enc.n_output_dims == 38
    np.testing.assert_allclose(out.numpy(), g["ide"], rtol=1e-5, atol=1e-5)
    out32 = IntegratedDirEncoding(4)(torch.from_numpy(g["xyz"]), torch.from_numpy(g["kappa_inv"]))
    np.testing.assert_allclose(out32.numpy(), g["ide"], rtol=1e-4, atol=1e-4)


def test_sdf_net_layout_query_and_struct(lib):
    """angelo_sdf_net_layout (a host-only call): the shapes the fused kernels
    are instantiated for, the forward's default of three products per layer,
    and the Python mirror's size matching the C struct's field layout (the
    last field sits after the 8-byte aligned block of offsets)."""
    from angelo_gb import _lib
    L = _lib.SdfNetLayout()
    assert lib.angelo_sdf_net_layout_query(16, 2, 65, ctypes.byref(L)) == 0
    assert (L.k_tiles1, L.n_hidden, L.n_tiles3, L.out_dim, L.mma_passes) == (3, 2, 9, 65, 3)
    assert L.bytes > 0 and L.off_tcw1 < L.off_tcw2 < L.off_tcw3 < L.bytes
    assert lib.angelo_sdf_net_layout_query(8, 1, 13, ctypes.byref(L)) == 0
    assert (L.k_tiles1, L.n_hidden, L.n_tiles3, L.mma_passes) == (2, 1, 2, 3)
    assert lib.angelo_sdf_net_layout_query(16, 3, 65, ctypes.byref(L)) != 0
    assert _lib.SdfNetLayout.mma_passes.offset == 5 * 4 + 4 + 8 * 8
    assert _lib.SdfNetLayout.operand_format.offset == 5 * 4 + 4 + 8 * 8 + 4
    assert ctypes.sizeof(_lib.SdfNetLayout) == 5 * 4 + 4 + 8 * 8 + 8
    assert L.operand_format == _lib.OPERAND_BF16


def test_probe_library_is_separate_and_complete(lib):
    """The tensor-core probes live in the test-only library
    (tests/native/tc_probe.h), not in the product library."""
    from native import build as probe
    txt = open(os.path.join(ROOT, "tests", "native", "tc_probe.h")).read()
    declared = sorted(set(re.findall(r"\b(angelo_[a-z0-9_]+)\s*\(", txt)))
    assert declared == sorted(probe.SIGNATURES)
    P = probe.load()
    for s in declared:
        assert hasattr(P, s), s
        assert not hasattr(lib, s), s


def test_backward_refuses_fp16_prepared_weights(lib):
    """The fused VolumeSDF backward reads bf16 operands: a weight buffer whose
    layout says fp16 (the precision form's forward buffer) is refused on the
    host, before anything is launched (the pointers here are host memory)."""
    import torch
    from angelo_gb import _lib
    L = _lib.SdfNetLayout()
    assert lib.angelo_sdf_net_layout_query(8, 1, 13, ctypes.byref(L)) == 0
    L.operand_format = _lib.OPERAND_FP16
    lay = _lib.HashGridLayout()
    desc = _lib.HashGridDesc(8, 2, 16, 16, 1.5)
    assert lib.angelo_hashgrid_layout(ctypes.byref(desc), ctypes.byref(lay)) == 0
    host = torch.zeros(64)
    p = host.data_ptr()
    rc = lib.angelo_sdf_stencil_bwd(ctypes.byref(lay), 8, p, 0, ctypes.byref(L), p, p, None, 1, 1.0,
                                    1e-2, 1, 0, p, p, None, None, None, 0, None, None, p, None)
    assert rc == _lib.ANGELO_E_INVALID
    assert b"operand_format" in lib.angelo_last_error_string()
    L.operand_format = 7
    rc = lib.angelo_sdf_stencil_fwd(ctypes.byref(lay), 8, p, 0, ctypes.byref(L), p, p, None, 1, 1.0,
                                    1e-2, 0, 0, 0, p, None, None, 0, None, p, None)
    assert rc == _lib.ANGELO_E_INVALID


def test_mlp_shape_queries(lib):
    """The fused VanillaMLP's size queries (host-only): supported shapes give
    the documented gradient layout, unsupported ones -1, and the fused forms
    route only MLPs of a supported shape to it."""
    from angelo_gb import fused
    from angelo_gb.network_utils import VanillaMLP
    for in_dim, nh, od in ((35, 1, 8), (19, 1, 8), (24, 2, 3), (64, 2, 16)):
        k1 = 16 * ((in_dim + 15) // 16)
        want = 64 * k1 + (64 * 64 + 64 if nh == 2 else 0) + 16 * 64 + 64 + 16
        assert lib.angelo_mlp_grad_size(in_dim, nh, od) == want
        assert lib.angelo_mlp_net_bytes(in_dim, nh, od) > 0
    for bad in ((0, 1, 8), (65, 1, 8), (35, 3, 8), (35, 0, 8), (35, 1, 17), (35, 1, 0)):
        assert lib.angelo_mlp_net_bytes(*bad) == -1
        assert lib.angelo_mlp_grad_size(*bad) == -1
    relu = dict(n_neurons=64, n_hidden_layers=1, activation="ReLU", output_activation="none")
    assert fused.mlp_supported(VanillaMLP(35, 8, relu))
    assert not fused.mlp_supported(VanillaMLP(35, 8, {**relu, "n_hidden_layers": 3}))
    assert not fused.mlp_supported(VanillaMLP(35, 8, {**relu, "output_activation": "sigmoid"}))
    assert not fused.mlp_supported(VanillaMLP(35, 8, {**relu, "n_neurons": 32}))
    assert not fused.mlp_supported(VanillaMLP(35, 13, {**relu, "sphere_init": True}))
    assert not fused.mlp_supported(VanillaMLP(80, 8, relu))


def test_serve_field_struct_matches_the_library(lib):
    """The ctypes mirror of angelo_serve_field has the C struct's size (a
    mismatch would hand the server shifted pointers)."""
    import ctypes as ct
    from angelo_gb import _lib
    assert ct.sizeof(_lib.ServeField) == lib.angelo_serve_field_bytes()
