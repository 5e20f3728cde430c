"""Fused forms of the hot path (libangelo_gb.so fused kernels).

* VolumeSDF: one kernel evaluates, per sample, the point, its 6-tap
  finite-difference stencil and the 6-tap curvature stencil (13 hash-grid +
  MLP evaluations, MLP on tensor cores in bf16x3) and writes sdf, grad,
  feature and laplace; the backward kernel recomputes the MLP activations from
  the stashed encodings and returns dL/dtable and dL/dW of every layer.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import call
from .ops import _p, _s, _table_dtype


SdfNetLayout = _lib.SdfNetLayout


def available():
    try:
        L = _lib.load()
    except RuntimeError:
        return False
    return hasattr(L, "angelo_sdf_stencil_fwd")


class SdfNet:
    """Prepared tensor-core operands of the geometry MLP (bf16 hi/lo fragments
    of every layer in forward and backward order, fp32 biases)."""

    def __init__(self, n_levels, n_hidden, out_dim, device):
        self.layout = SdfNetLayout()
        call("angelo_sdf_net_layout_query", n_levels, n_hidden, out_dim, ctypes.byref(self.layout))
        self.n_levels, self.n_hidden, self.out_dim = n_levels, n_hidden, out_dim
        self.buf = torch.empty(self.layout.bytes, dtype=torch.uint8, device=device)
        self.grad_size = _lib.raw("angelo_sdf_grad_size")(ctypes.byref(self.layout))
        self.k1cols = 16 * self.layout.k_tiles1
        self.out_pad = 16 * self.layout.k_tiles3b

    def prepare(self, Ws):
        """Ws: [(W, b)] fp32 effective weights of the VanillaMLP layers."""
        W1, b1 = Ws[0]
        W2, b2 = Ws[1] if self.n_hidden == 2 else (None, None)
        W3, b3 = Ws[-1]
        ts = [t.detach().float().contiguous() if t is not None else None
              for t in (W1, b1, W2, b2, W3, b3)]
        call("angelo_sdf_prep", ctypes.byref(self.layout), self.n_levels, W1.shape[1],
             *[_p(t) for t in ts], _p(self.buf), _s(self.buf.device))
        return ts

    def unpack_grads(self, g, in_dim):
        """Kernel-order flat gradient -> reference-order (dW, db) per layer."""
        L2 = 2 * self.n_levels
        k1 = self.k1cols
        o = 0
        dW1k = g[o:o + 64 * k1].view(64, k1)
        o += 64 * k1
        dW2 = g[o:o + 64 * 64].view(64, 64)
        o += 64 * 64
        dW3 = g[o:o + self.out_pad * 64].view(self.out_pad, 64)[: self.out_dim]
        o += self.out_pad * 64
        db1 = g[o:o + 64]
        db2 = g[o + 64:o + 128]
        db3 = g[o + 128:o + 128 + self.out_pad][: self.out_dim]
        dW1 = torch.cat([dW1k[:, L2:L2 + 3], dW1k[:, :L2]], dim=1)[:, :in_dim]
        out = [(dW1, db1)]
        if self.n_hidden == 2:
            out.append((dW2, db2))
        out.append((dW3, db3))
        return out


class _FusedSdf(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, rand_dirs, table, meta, *weights):
        geom, net, flags = meta["geom"], meta["net"], meta["flags"]
        with_grad, with_laplace, with_feature = flags
        Ws = [(weights[2 * i], weights[2 * i + 1]) for i in range(len(weights) // 2)]
        net.prepare(Ws)
        spec = geom.hashgrid.encoding.spec
        active = geom.hashgrid.mask_levels
        S = pos.shape[0]
        dev = pos.device
        od = net.out_dim
        sdf = torch.empty(S, device=dev)
        grad = torch.empty(S, 3, device=dev) if with_grad else None
        feature = torch.empty(S, od + 3, device=dev) if with_feature else None
        lap = torch.empty(S, 1, device=dev) if with_laplace else None
        training = any(ctx.needs_input_grad[2:])
        stash_x = torch.empty(S, 13, 36, device=dev) if training else None
        stash_s = torch.empty(S, 13, device=dev) if training else None
        rd = rand_dirs.contiguous() if rand_dirs is not None else None
        call("angelo_sdf_stencil_fwd", ctypes.byref(spec.layout), int(active), _p(table),
             _table_dtype(table), ctypes.byref(net.layout), _p(net.buf), _p(pos), _p(rd), S,
             float(geom.radius), float(geom._finite_difference_eps or 1.0), int(with_grad),
             int(with_laplace), int(with_feature), _p(sdf), _p(grad), _p(feature),
             od + 3, _p(lap), _p(stash_x), _p(stash_s), _s(dev),
             units=dict(n=S, od=net.out_dim, evals=13 if with_laplace else (7 if with_grad else 1),
                        active=int(active), tbytes=table.element_size(), train=training))
        ctx.meta = meta
        ctx.in_dim = weights[0].shape[1]
        ctx.n_w = len(weights)
        if training:
            ctx.save_for_backward(pos, rd, table, stash_x, stash_s)
        outs = [sdf, grad, feature, lap]
        return tuple(t if t is not None else torch.empty(0, device=dev) for t in outs)

    @staticmethod
    def backward(ctx, g_sdf, g_grad, g_feat, g_lap):
        pos, rd, table, stash_x, stash_s = ctx.saved_tensors
        geom, net, flags = ctx.meta["geom"], ctx.meta["net"], ctx.meta["flags"]
        with_grad, with_laplace, with_feature = flags
        spec = geom.hashgrid.encoding.spec
        active = geom.hashgrid.mask_levels
        S = pos.shape[0]
        dev = pos.device
        need_table = ctx.needs_input_grad[2]
        d_table = torch.zeros(spec.n_params, device=dev) if need_table else None
        d_net = torch.zeros(net.grad_size, device=dev)

        def c(t, shape_ok):
            return t.contiguous().float() if (t is not None and shape_ok) else None
        gs = c(g_sdf, g_sdf is not None and g_sdf.numel() == S)
        gg = c(g_grad, with_grad and g_grad is not None and g_grad.numel() == 3 * S)
        gf = c(g_feat, with_feature and g_feat is not None and g_feat.numel() > 0)
        gl = c(g_lap, with_laplace and g_lap is not None and g_lap.numel() == S)
        call("angelo_sdf_stencil_bwd", ctypes.byref(spec.layout), int(active), _p(table),
             _table_dtype(table), ctypes.byref(net.layout), _p(net.buf), _p(pos), _p(rd), S,
             float(geom.radius), float(geom._finite_difference_eps or 1.0), int(with_grad),
             int(with_laplace), _p(stash_x), _p(stash_s), _p(gs), _p(gg), _p(gf),
             gf.stride(0) if gf is not None else 0, _p(gl), _p(d_table), _p(d_net), _s(dev),
             units=dict(n=S, od=net.out_dim, evals=13 if with_laplace else (7 if with_grad else 1),
                        active=int(active), tbytes=table.element_size(), train=True))
        grads = net.unpack_grads(d_net, ctx.in_dim)
        flat = []
        for dW, db in grads:
            flat += [dW, db]
        return (None, None, d_table, None, *flat)


def _net_for(geom):
    net = getattr(geom, "_fused_net", None)
    mlp = geom.network
    if net is None or net.buf.device != geom.hashgrid.encoding.params.device:
        net = SdfNet(geom.hashgrid.n_level, mlp.n_hidden_layers, geom.n_output_dims,
                     geom.hashgrid.encoding.params.device)
        geom._fused_net = net
    return net


def volume_sdf_forward(geom, points, with_grad, with_feature, with_laplace):
    """VolumeSDF.forward in one fused kernel (see the module docstring)."""
    if with_laplace and not with_grad:
        raise ValueError("with_laplace needs with_grad")
    net = _net_for(geom)
    pos = points.reshape(-1, 3).float().contiguous()
    rd = None
    if with_laplace:
        pts_c = (pos - (-geom.radius)) / (geom.radius - (-geom.radius))
        rd = geom.curvature_dirs_fn(pts_c).float().contiguous()
    weights = []
    for W, b in geom.network.effective_weights():
        weights += [W, b]
    table = geom.hashgrid.encoding.params
    meta = dict(geom=geom, net=net, flags=(bool(with_grad), bool(with_laplace),
                                           bool(with_feature)))
    with torch.set_grad_enabled(geom.training and torch.is_grad_enabled()):
        sdf, grad, feature, lap = _FusedSdf.apply(pos, rd, table, meta, *weights)
    shp = points.shape[:-1]
    rv = [sdf.view(*shp)]
    if with_grad:
        rv.append(grad.view(*shp, 3))
    if with_feature:
        rv.append(feature.view(*shp, -1))
    if with_laplace:
        rv.append(lap.view(*shp, 1))
    return rv


def sdf_query(geom, points):
    """forward_level: SDF only, one evaluation per point."""
    return volume_sdf_forward(geom, points, False, False, False)[0]
