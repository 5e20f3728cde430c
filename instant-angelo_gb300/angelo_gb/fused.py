"""Fused forms of the hot path (libangelo_gb.so fused kernels).

* VolumeSDF: per sample the point, its 6-tap finite-difference stencil and
  the 6-tap curvature stencil (13 hash-grid + MLP evaluations): a
  shared-gather stencil encode per (sample, level), the MLP on tensor cores
  in bf16x3 with the stencil arithmetic fused, and in the backward the MLP
  recomputed from the kept encodings, dL/dW as a per-CTA staged GEMM and a
  shared-corner scatter of dL/dtable (the curvature taps also carry the hash
  grid's positional derivative).
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

    def __init__(self, n_levels, n_hidden, out_dim, device, operand_format=_lib.OPERAND_BF16):
        self.layout = SdfNetLayout()
        call("angelo_sdf_net_layout_query", n_levels, n_hidden, out_dim, ctypes.byref(self.layout))
        self.layout.operand_format = int(operand_format)
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


def workspace_floats(spec, n, with_grad, with_laplace, backward):
    """Floats of the fused VolumeSDF forward (backward=False) or backward
    workspace for n samples."""
    k = _lib.raw("angelo_sdf_workspace_floats")(ctypes.byref(spec.layout), int(n), int(with_grad),
                                                 int(with_laplace), int(backward))
    if k < 0:
        raise ValueError("angelo_sdf_workspace_floats: invalid arguments")
    return k


class _FusedSdf(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, rand_dirs, table, meta, *weights):
        geom, net, flags = meta["geom"], meta["net"], meta["flags"]
        with_grad, with_laplace, with_feature = flags
        Ws = [(weights[2 * i], weights[2 * i + 1]) for i in range(len(weights) // 2)]
        training = any(ctx.needs_input_grad[2:])
        # the forward's operands (fp16 in the fp16 precision form); the
        # backward always reads the bf16 buffer
        fnet = meta.get("net_fwd", net)
        if not meta.get("prepared"):
            fnet.prepare(Ws)
        if training and fnet is not net:
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
        work = torch.empty(workspace_floats(spec, S, with_grad, with_laplace, False), device=dev)
        rd = rand_dirs.contiguous() if rand_dirs is not None else None
        n_ev = 13 if with_laplace else (7 if with_grad else 1)
        # the table the encode gathers from (an fp16 copy in the fp16-table form)
        table = meta.get("table_fwd", table)
        call("angelo_sdf_stencil_fwd", ctypes.byref(spec.layout), int(active), _p(table),
             _table_dtype(table), ctypes.byref(fnet.layout), _p(fnet.buf), _p(pos), _p(rd), S,
             float(geom.radius), float(geom._finite_difference_eps or 1.0), int(with_grad),
             int(with_laplace), int(with_feature), _p(sdf), _p(grad), _p(feature),
             od + 3, _p(lap), _p(work), _s(dev),
             launches=4 if with_laplace else 2,
             units=dict(n=S, od=net.out_dim, evals=n_ev, active=int(active),
                        levels=spec.layout.n_levels, tbytes=table.element_size(), train=training))
        ctx.meta = meta
        ctx.in_dim = weights[0].shape[1]
        ctx.n_w = len(weights)
        if training:
            ctx.save_for_backward(pos, rd, table, work)
        outs = [sdf, grad, feature, lap]
        return tuple(t if t is not None else torch.empty(0, device=dev) for t in outs)

    @staticmethod
    def backward(ctx, g_sdf, g_grad, g_feat, g_lap):
        pos, rd, table, work = ctx.saved_tensors
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
        bwork = torch.empty(workspace_floats(spec, S, with_grad, with_laplace, True), device=dev)
        n_ev = 13 if with_laplace else (7 if with_grad else 1)
        call("angelo_sdf_stencil_bwd", ctypes.byref(spec.layout), int(active), _p(table),
             _table_dtype(table), ctypes.byref(net.layout), _p(net.buf), _p(pos), _p(rd), S,
             float(geom.radius), float(geom._finite_difference_eps or 1.0), int(with_grad),
             int(with_laplace), _p(work), _p(bwork), _p(gs), _p(gg), _p(gf),
             gf.stride(0) if gf is not None else 0, _p(gl), _p(d_table), _p(d_net), _s(dev),
             launches=3 if with_laplace else 2,
             units=dict(n=S, od=net.out_dim, evals=n_ev, active=int(active),
                        levels=spec.layout.n_levels, tbytes=table.element_size(), train=True))
        grads = net.unpack_grads(d_net, ctx.in_dim)
        flat = []
        for dW, db in grads:
            flat += [dW, db]
        return (None, None, d_table, None, *flat)


class _WeightNorm(torch.autograd.Function):
    """W_i = g_i * v_i / ||v_i||_row for every layer in one launch, and the
    backward in one launch (angelo_weight_norm_fwd/bwd)."""

    @staticmethod
    def forward(ctx, *vg):
        vs = [t.detach().float().contiguous() for t in vg[0::2]]
        gs = [t.detach().float().contiguous() for t in vg[1::2]]
        n = len(vs)
        ws = [torch.empty_like(v) for v in vs]
        rows = (ctypes.c_int32 * n)(*[v.shape[0] for v in vs])
        cols = (ctypes.c_int32 * n)(*[v.shape[1] for v in vs])
        ptrs = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
        call("angelo_weight_norm_fwd", n, rows, cols, ptrs(vs), ptrs(gs), ptrs(ws), _s(vs[0].device))
        ctx.save_for_backward(*vs, *gs)
        ctx.n = n
        return tuple(ws)

    @staticmethod
    def backward(ctx, *dws):
        n = ctx.n
        vs, gs = ctx.saved_tensors[:n], ctx.saved_tensors[n:]
        dws = [d.float().contiguous() if d is not None else torch.zeros_like(v) for d, v in zip(dws, vs)]
        dvs = [torch.empty_like(v) for v in vs]
        dgs = [torch.empty_like(g) for g in gs]
        rows = (ctypes.c_int32 * n)(*[v.shape[0] for v in vs])
        cols = (ctypes.c_int32 * n)(*[v.shape[1] for v in vs])
        ptrs = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
        call("angelo_weight_norm_bwd", n, rows, cols, ptrs(vs), ptrs(gs), ptrs(dws), ptrs(dvs),
             ptrs(dgs), _s(vs[0].device))
        out = []
        for dv, dg in zip(dvs, dgs):
            out += [dv, dg]
        return tuple(out)


def effective_weights(mlp):
    """[(W, b)] of a VanillaMLP: weight-normalised layers through the native
    weight norm (one launch forward, one backward), plain layers as they are."""
    from .network_utils import WNLinear
    lins = mlp.linears()
    wn = [m for m in lins if isinstance(m, WNLinear)]
    if not wn or len(wn) > 8 or not wn[0].weight_v.is_cuda:
        return mlp.effective_weights()
    vg = []
    for m in wn:
        vg += [m.weight_v, m.weight_g]
    ws = iter(_WeightNorm.apply(*vg))
    return [(next(ws) if isinstance(m, WNLinear) else m.weight, m.bias) for m in lins]


# fused_precision of the drop-in config: "fp32" (the default: bf16x3 operands,
# fp32 accumulation), "bf16" (one bf16 pass per forward layer) or "fp16"
# (one fp16 pass per forward layer: the precision form); the backward is
# bf16x3 in every form
PRECISIONS = ("fp32", "bf16", "fp16")


def _precision(mod):
    p = getattr(mod, "fused_precision", "fp32")
    if p not in PRECISIONS:
        raise ValueError(f"fused_precision {p!r}: one of {PRECISIONS}")
    return p


def _net_for(geom, operand_format=_lib.OPERAND_BF16):
    attr = "_fused_net" if operand_format == _lib.OPERAND_BF16 else "_fused_net_fp16"
    net = getattr(geom, attr, None)
    mlp = geom.network
    if net is None or net.buf.device != geom.hashgrid.encoding.params.device:
        net = SdfNet(geom.hashgrid.n_level, mlp.n_hidden_layers, geom.n_output_dims,
                     geom.hashgrid.encoding.params.device, operand_format)
        setattr(geom, attr, net)
    return net


def prepare_ahead(model):
    """The training step's weight preparation, enqueued before the march
    reads its sample count on the host: the geometry MLP's effective weights
    (the native weight norm) and both networks' tensor-core operands.  The
    next fused VolumeSDF and radiance calls take them as they are, so the
    host has less to enqueue between that read and the forward's kernels.
    Only the default form (fp32 table, bf16x3 operands) is prepared ahead."""
    geom, tex = model.geometry, model.texture
    if (_precision(geom) != "fp32" or getattr(geom, "fused_table_dtype", "fp32") != "fp32"
            or geom.hashgrid.encoding.params.dtype != torch.float32):
        return
    net = _net_for(geom)
    net.layout.mma_passes = 3
    Ws = effective_weights(geom.network)
    net.prepare(Ws)
    geom._ahead = (Ws, net)
    if (type(tex).__name__ in ("VolumeRadiance", "VolumeDualColor") and _precision(tex) == "fp32"
            and tex.config.get("color_activation") == "sigmoid"):
        rnet = getattr(tex, "_fused_net", None)
        F_ = geom.n_output_dims + 3
        if rnet is None or rnet.feat_dim != F_ or rnet.buf.device != geom.hashgrid.encoding.params.device:
            rnet = RadNet(F_, geom.hashgrid.encoding.params.device)
            tex._fused_net = rnet
        RW = tex.network.effective_weights()
        rnet.prepare(RW)
        tex._ahead = (RW, rnet)


def volume_sdf_forward(geom, points, with_grad, with_feature, with_laplace):
    """VolumeSDF.forward in one fused kernel (see the module docstring)."""
    if with_laplace and not with_grad:
        raise ValueError("with_laplace needs with_grad")
    net = _net_for(geom)
    pos = points.reshape(-1, 3).float().contiguous()
    rd = None
    if with_laplace:
        if geom.curvature_dirs_fn is torch.randn_like:
            # the same draws as randn_like of the contracted points (shape,
            # dtype and device are all it reads)
            rd = torch.randn_like(pos)
        else:
            pts_c = (pos - (-geom.radius)) / (geom.radius - (-geom.radius))
            rd = geom.curvature_dirs_fn(pts_c).float().contiguous()
    ahead = getattr(geom, "_ahead", None)
    geom._ahead = None
    weights = []
    for W, b in (ahead[0] if ahead is not None and ahead[1] is net else effective_weights(geom.network)):
        weights += [W, b]
    table = geom.hashgrid.encoding.params
    prec = _precision(geom)
    table_fwd = None
    if getattr(geom, "fused_table_dtype", "fp32") == "fp16" and table.dtype == torch.float32:
        table_fwd = table.detach().half()
    net.layout.mma_passes = 1 if prec == "bf16" else 3
    meta = dict(geom=geom, net=net, flags=(bool(with_grad), bool(with_laplace),
                                           bool(with_feature)),
                prepared=ahead is not None and ahead[1] is net and prec == "fp32")
    if prec == "fp16":
        fnet = _net_for(geom, _lib.OPERAND_FP16)
        fnet.layout.mma_passes = 1
        meta["net_fwd"] = fnet
    if table_fwd is not None:
        meta["table_fwd"] = table_fwd
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


# ------------------------------------------------------------ VanillaMLP (ReLU)


class MlpNet:
    """Prepared tensor-core operands of a ReLU VanillaMLP (one or two hidden
    layers of 64, no output activation): angelo_mlp_prep's buffer."""

    def __init__(self, in_dim, n_hidden, out_dim, device):
        self.in_dim, self.n_hidden, self.out_dim = int(in_dim), int(n_hidden), int(out_dim)
        nbytes = _lib.raw("angelo_mlp_net_bytes")(self.in_dim, self.n_hidden, self.out_dim)
        if nbytes < 0:
            raise ValueError(f"MLP {in_dim} -> {n_hidden} x 64 -> {out_dim} not supported by the "
                             "fused kernel")
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
        self.grad_size = _lib.raw("angelo_mlp_grad_size")(self.in_dim, self.n_hidden, self.out_dim)
        self.k1cols = 16 * ((self.in_dim + 15) // 16)

    def key(self):
        return (self.in_dim, self.n_hidden, self.out_dim, self.buf.device)

    def prepare(self, Ws):
        ts = [t.detach().float().contiguous() for W, b in Ws for t in (W, b)]
        if self.n_hidden == 1:
            ts = ts[:2] + [None, None] + ts[2:]
        call("angelo_mlp_prep", self.in_dim, self.n_hidden, self.out_dim, *[_p(t) for t in ts],
             _p(self.buf), _s(self.buf.device))

    def unpack_grads(self, g):
        k1, o = self.k1cols, 0
        dW1 = g[o:o + 64 * k1].view(64, k1)[:, :self.in_dim]
        o += 64 * k1
        dW2 = None
        if self.n_hidden == 2:
            dW2 = g[o:o + 4096].view(64, 64)
            o += 4096
        dW3 = g[o:o + 16 * 64].view(16, 64)[:self.out_dim]
        o += 16 * 64
        db1 = g[o:o + 64]
        o += 64
        db2 = None
        if self.n_hidden == 2:
            db2 = g[o:o + 64]
            o += 64
        db3 = g[o:o + self.out_dim]
        out = [(dW1, db1)] + ([(dW2, db2)] if self.n_hidden == 2 else []) + [(dW3, db3)]
        return out


class _FusedMlp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, net, *weights):
        Ws = [(weights[2 * i], weights[2 * i + 1]) for i in range(len(weights) // 2)]
        net.prepare(Ws)
        x = x.contiguous().float()
        n = x.shape[0]
        out = torch.empty(n, net.out_dim, device=x.device)
        call("angelo_mlp_fused_fwd", net.in_dim, net.n_hidden, net.out_dim, _p(net.buf), _p(x),
             x.stride(0), n, _p(out), out.stride(0), _s(x.device),
             units=dict(n=n, in_dim=net.in_dim, n_hidden=net.n_hidden, out_dim=net.out_dim, bwd=False))
        ctx.save_for_backward(x)
        ctx.net = net
        return out

    @staticmethod
    def backward(ctx, g_out):
        (x,) = ctx.saved_tensors
        net = ctx.net
        n = x.shape[0]
        g_out = g_out.contiguous().float()
        d_x = torch.empty_like(x) if ctx.needs_input_grad[0] else None
        d_net = torch.zeros(net.grad_size, device=x.device)
        call("angelo_mlp_fused_bwd", net.in_dim, net.n_hidden, net.out_dim, _p(net.buf), _p(x),
             x.stride(0), None, n, _p(g_out), g_out.stride(0), _p(d_x),
             d_x.stride(0) if d_x is not None else 0, _p(d_net), _s(x.device),
             units=dict(n=n, in_dim=net.in_dim, n_hidden=net.n_hidden, out_dim=net.out_dim, bwd=True))
        flat = []
        for dW, db in net.unpack_grads(d_net):
            flat += [dW, db]
        return (d_x, None, *flat)


def mlp_supported(mlp):
    """Whether a VanillaMLP has the shape the fused kernel runs: ReLU hidden
    layers of 64 (no sphere init, no weight norm), one or two of them, no
    output activation, in <= 64, out <= 16."""
    return (not mlp.sphere_init and not mlp.weight_norm and mlp.n_neurons == 64
            and mlp.n_hidden_layers in (1, 2) and mlp.output_activation in (None, "none", "None")
            and 1 <= mlp.dim_in <= 64 and 1 <= mlp.dim_out <= 16)


def mlp_forward(mlp, x):
    """VanillaMLP.forward on the fused kernel (models/network_utils.py:134-140)."""
    net = getattr(mlp, "_fused_net", None)
    if net is None or net.key() != (mlp.dim_in, mlp.n_hidden_layers, mlp.dim_out, x.device):
        net = MlpNet(mlp.dim_in, mlp.n_hidden_layers, mlp.dim_out, x.device)
        mlp._fused_net = net
    weights = []
    for W, b in mlp.effective_weights():
        weights += [W, b]
    return _FusedMlp.apply(x, net, *weights)


class _ReusedDensityField(torch.autograd.Function):
    """The density field's MLP output on samples whose encodings X and
    outputs a no-grad pass already computed (the learned background's
    visibility test evaluates every marched sample; the kept ones are
    evaluated again by the reference, with bit-identical results here).  The
    forward hands the kept outputs on; the backward runs the MLP backward
    from the kept encodings and scatters dL/dX into the hash table."""

    @staticmethod
    def forward(ctx, pts, X, rows, out, table, meta, *weights):
        ctx.save_for_backward(pts, X, rows, table)
        ctx.meta = meta
        return out.clone()

    @staticmethod
    def backward(ctx, g_out):
        pts, X, rows, table = ctx.saved_tensors
        net, spec, active, xyz = ctx.meta["net"], ctx.meta["spec"], ctx.meta["active"], ctx.meta["xyz"]
        n = rows.shape[0]
        g = g_out.contiguous().float()
        dX = torch.empty(n, X.shape[1], device=X.device)
        d_net = torch.zeros(net.grad_size, device=X.device)
        # the kept rows' encodings are read in place from the visibility
        # pass's X through their row indices
        call("angelo_mlp_fused_bwd", net.in_dim, net.n_hidden, net.out_dim, _p(net.buf), _p(X),
             X.stride(0), _p(rows), n, _p(g), g.stride(0), _p(dX), dX.stride(0), _p(d_net), _s(X.device),
             units=dict(n=n, in_dim=net.in_dim, n_hidden=net.n_hidden, out_dim=net.out_dim, bwd=True))
        dtable = None
        need_table = ctx.needs_input_grad[4]
        if need_table and active > 0:
            dtable = torch.zeros(spec.n_params, device=X.device, dtype=torch.float32)
            call("angelo_hashgrid_bwd", ctypes.byref(spec.layout), int(active), _p(pts), n, _p(table),
                 _table_dtype(table), int(xyz), _p(dX), dX.stride(0), 0, _p(dtable), None, _s(X.device),
                 units=dict(n=n, active=int(active), L=spec.n_levels, tbytes=table.element_size(),
                            dtable=True, dx=False))
        elif need_table:
            dtable = torch.zeros(spec.n_params, device=X.device, dtype=torch.float32)
        flat = []
        for dW, db in net.unpack_grads(d_net):
            flat += [dW, db]
        return (None, None, None, None, dtable, None, *flat)


def density_field_reused(geom, pts, X, rows, out):
    """VolumeDensity's (density, feature) on kept samples from the visibility
    pass: their contracted points and MLP outputs, and the visibility pass's
    encodings X of every sample with the kept rows' indices (see
    _ReusedDensityField); differentiable w.r.t. the hash table and the MLP."""
    enc, mlp = geom.encoding_with_network.encoding, geom.encoding_with_network.network
    grid = enc.encoding
    net = mlp._fused_net
    weights = []
    for W, b in mlp.effective_weights():
        weights += [W, b]
    meta = dict(net=net, spec=grid.encoding.spec, active=int(grid.mask_levels), xyz=bool(enc.include_xyz))
    o = _ReusedDensityField.apply(pts.contiguous(), X.contiguous(), rows.to(torch.int32).contiguous(),
                                  out.contiguous(), grid.encoding.params, meta, *weights)
    return geom.outputs(o)


class _DensityComposite(torch.autograd.Function):
    """The learned background's weights from density, accumulation and
    background blend in one kernel each way (angelo_density_composite_*)."""

    @staticmethod
    def forward(ctx, sigma, rgb, t0, t1, offsets, bg):
        n_rays = offsets.numel() - 1
        S = sigma.numel()
        dev = sigma.device
        sigma, rgb = sigma.contiguous().float(), rgb.contiguous().float()
        t0, t1, bg = t0.contiguous(), t1.contiguous(), bg.contiguous().float()
        opacity = torch.empty(n_rays, 1, device=dev)
        depth = torch.empty(n_rays, 1, device=dev)
        comp = torch.empty(n_rays, 3, device=dev)
        weights = torch.empty(S, device=dev)
        trans = torch.empty(S, device=dev)
        call("angelo_density_composite_fwd", _p(offsets), n_rays, _p(sigma), _p(t0), _p(t1), _p(rgb),
             _p(bg), _p(opacity), _p(depth), _p(comp), _p(weights), _p(trans), _s(dev),
             units=dict(n=S, rays=n_rays, bwd=False))
        ctx.save_for_backward(sigma, rgb, t0, t1, offsets, bg, weights, trans)
        ctx.mark_non_differentiable(weights)
        ctx.set_materialize_grads(False)
        return comp, opacity, depth, weights

    @staticmethod
    def backward(ctx, g_comp, g_op, g_depth, g_w):
        sigma, rgb, t0, t1, offsets, bg, weights, trans = ctx.saved_tensors
        n_rays = offsets.numel() - 1
        dev = sigma.device

        def c(t):
            return t.contiguous().float() if t is not None else None
        d_sigma = torch.empty_like(sigma)
        d_rgb = torch.empty_like(rgb)
        call("angelo_density_composite_bwd", _p(offsets), n_rays, _p(sigma), _p(t0), _p(t1), _p(rgb),
             _p(bg), _p(weights), _p(trans), _p(c(g_op)), _p(c(g_depth)), _p(c(g_comp)), _p(d_sigma),
             _p(d_rgb), _s(dev), units=dict(n=sigma.numel(), rays=n_rays, bwd=True))
        return d_sigma, d_rgb, None, None, None, None


def density_composite(sigma, rgb, t0, t1, offsets, bg):
    """(comp_rgb with bg blended, opacity, depth, weights) of the learned
    background (models/neus.py:171-177)."""
    return _DensityComposite.apply(sigma.reshape(-1), rgb, t0.reshape(-1), t1.reshape(-1), offsets, bg)


def sample_points(rays_o, rays_d, ri, t0, t1):
    """(world points (S, 3), midpoints (S,)) of the marched samples in one
    launch (angelo_sample_points), bit-identical to
    rays_o[ri] + rays_d[ri] * ((t0 + t1) * 0.5)[:, None]."""
    n = t0.numel()
    pts = torch.empty(n, 3, device=t0.device)
    mid = torch.empty(n, device=t0.device)
    call("angelo_sample_points", _p(rays_o), _p(rays_d), _p(ri), _p(t0), _p(t1), n, _p(pts), _p(mid),
         _s(t0.device), units=dict(n=n))
    return pts, mid


def bg_points(rays_o, rays_d, ri, t0, t1, radius):
    """The learned background's samples as contracted points (angelo_bg_points)."""
    n = t0.numel()
    pts = torch.empty(n, 3, device=t0.device)
    call("angelo_bg_points", _p(rays_o), _p(rays_d), _p(ri), _p(t0), _p(t1), n, float(radius), _p(pts),
         _s(t0.device), units=dict(n=n))
    return pts


def bg_visible(out, density_bias, ri, t0, t1, offsets, pts, eps=1e-4):
    """nerfacc's visibility test on the background's samples from the density
    MLP's output (density exp(out0 + bias)): the kept prefix of every ray,
    compacted.  Returns (ray indices, t0, t1, points, outputs, their rows in
    the inputs, offsets); one device read (the kept count)."""
    n_rays = offsets.numel() - 1
    dev = t0.device
    if t0.numel() >= 1 << 31:
        raise ValueError("bg_visible: the kept rows are int32 indices (fewer than 2^31 samples)")
    kept = torch.empty(n_rays, dtype=torch.int32, device=dev)
    call("angelo_bg_visibility", _p(out), out.stride(0), float(density_bias), _p(t0), _p(t1), _p(offsets),
         n_rays, float(eps), _p(kept), _s(dev), units=dict(rays=n_rays))
    koff = torch.empty(n_rays + 1, dtype=torch.int64, device=dev)
    ws = torch.empty(_lib.raw("angelo_scan_workspace_size")(n_rays), dtype=torch.uint8, device=dev)
    call("angelo_scan", _p(kept), n_rays, _p(koff), _p(ws), _s(dev))
    total = int(koff[n_rays].item())
    od = out.shape[1]
    ri_k = torch.empty(total, dtype=torch.int32, device=dev)
    t0_k = torch.empty(total, device=dev)
    t1_k = torch.empty(total, device=dev)
    pts_k = torch.empty(total, 3, device=dev)
    out_k = torch.empty(total, od, device=dev)
    rows = torch.empty(total, dtype=torch.int32, device=dev)
    call("angelo_bg_compact", _p(offsets), _p(kept), _p(koff), n_rays, _p(ri), _p(t0), _p(t1), _p(pts),
         _p(out.contiguous()), od, _p(ri_k), _p(t0_k), _p(t1_k), _p(pts_k), _p(out_k), _p(rows), _s(dev),
         units=dict(rays=n_rays, n=total))
    return ri_k, t0_k, t1_k, pts_k, out_k, rows, koff


# ----------------------------------------------------------------- radiance


class RadNet:
    """Prepared tensor-core operands of a 2-hidden-layer ReLU radiance MLP
    (VolumeRadiance / VolumeDualColor, models/texture.py:10-64)."""

    def __init__(self, feat_dim, device, operand_format=_lib.OPERAND_BF16):
        self.feat_dim = int(feat_dim)
        self.operand_format = int(operand_format)
        nbytes = _lib.raw("angelo_radiance_net_bytes")(self.feat_dim)
        if nbytes < 0:
            raise ValueError(f"radiance feature width {feat_dim} not supported by the fused kernel")
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
        self.grad_size = _lib.raw("angelo_radiance_grad_size")(self.feat_dim)
        self.in_dim = self.feat_dim + 19
        self.k1cols = 16 * ((self.in_dim + 15) // 16)

    def prepare(self, Ws):
        ts = [t.detach().float().contiguous() for W, b in Ws for t in (W, b)]
        call("angelo_radiance_prep_format", self.feat_dim, self.operand_format,
             *[_p(t) for t in ts], _p(self.buf), _s(self.buf.device))

    def unpack_grads(self, g):
        k1 = self.k1cols
        o = 0
        dW1 = g[o:o + 64 * k1].view(64, k1)[:, :self.in_dim]
        o += 64 * k1
        dW2 = g[o:o + 4096].view(64, 64)
        o += 4096
        dW3 = g[o:o + 16 * 64].view(16, 64)[:3]
        o += 16 * 64
        return [(dW1, g[o:o + 64]), (dW2, g[o + 64:o + 128]), (dW3, g[o + 128:o + 131])]


class _FusedRadiance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, feature, grad, ray_idx, rays_d, meta, *weights):
        net, dual = meta["net"], meta["dual"]
        Ws = [(weights[2 * i], weights[2 * i + 1]) for i in range(3)]
        fnet = meta.get("net_fwd", net)
        if not meta.get("prepared"):
            fnet.prepare(Ws)
        if fnet is not net and any(ctx.needs_input_grad):
            net.prepare(Ws)
        feature = feature.contiguous()
        grad = grad.contiguous() if grad is not None else None
        S = feature.shape[0]
        rgb = torch.empty(S, 3, device=feature.device)
        flags = int(dual) | (2 if meta.get("one_pass") else 0) | \
            (4 if fnet.operand_format == _lib.OPERAND_FP16 else 0)
        call("angelo_radiance_fwd", net.feat_dim, _p(fnet.buf), _p(feature), feature.stride(0),
             _p(grad), _p(ray_idx), _p(rays_d), S, flags, _p(rgb), _s(feature.device),
             units=dict(n=S, F=net.feat_dim, bwd=False))
        ctx.save_for_backward(feature, grad, ray_idx, rays_d)
        ctx.meta = meta
        return rgb

    @staticmethod
    def backward(ctx, g_rgb):
        feature, grad, ray_idx, rays_d = ctx.saved_tensors
        net, dual = ctx.meta["net"], ctx.meta["dual"]
        S = feature.shape[0]
        g_rgb = g_rgb.contiguous().float()
        # the kernel writes every column of every row
        d_feature = torch.empty_like(feature)
        d_grad = torch.empty_like(grad) if grad is not None else None
        d_net = torch.zeros(net.grad_size, device=feature.device)
        call("angelo_radiance_bwd", net.feat_dim, _p(net.buf), _p(feature), feature.stride(0),
             _p(grad), _p(ray_idx), _p(rays_d), S, int(dual), _p(g_rgb), _p(d_feature),
             _p(d_grad), _p(d_net), _s(feature.device),
             units=dict(n=S, F=net.feat_dim, bwd=True))
        flat = []
        for dW, db in net.unpack_grads(d_net):
            flat += [dW, db]
        return (d_feature, d_grad, None, None, None, *flat)


def radiance_forward(texture, feature, grad, ray_idx, rays_d):
    """The radiance network on the fused kernel; grad None: a VolumeRadiance
    without a normal input (the learned background's texture, input
    [feature, SH4]), whose first layer gets three zero columns where the
    kernel stages the normal."""
    net = getattr(texture, "_fused_net", None)
    F_ = feature.shape[-1]
    if net is None or net.feat_dim != F_ or net.buf.device != feature.device:
        net = RadNet(F_, feature.device)
        texture._fused_net = net
    ahead = getattr(texture, "_ahead", None)
    texture._ahead = None
    use_ahead = ahead is not None and ahead[1] is net and grad is not None
    weights = []
    for W, b in (ahead[0] if use_ahead else texture.network.effective_weights()):
        weights += [W, b]
    if grad is None:
        if weights[0].shape[1] != F_ + 16:
            raise ValueError("a radiance network without a normal input takes [feature, SH4]")
        weights[0] = torch.nn.functional.pad(weights[0], (0, 3))
    prec = _precision(texture)
    meta = dict(net=net, dual=bool(getattr(texture, "dual", False)), one_pass=prec in ("bf16", "fp16"),
                prepared=use_ahead and prec == "fp32")
    if prec == "fp16":
        fnet = getattr(texture, "_fused_net_fp16", None)
        if fnet is None or fnet.feat_dim != F_ or fnet.buf.device != feature.device:
            fnet = RadNet(F_, feature.device, _lib.OPERAND_FP16)
            texture._fused_net_fp16 = fnet
        meta["net_fwd"] = fnet
    return _FusedRadiance.apply(feature, grad, ray_idx, rays_d, meta, *weights)


# --------------------------------------------------------------- compositing

FP64_ALPHA_GATE = 2048.0
# the fused radiance / compositing kernels are used by neus_forward when set
FUSED_RENDER = True


class _FusedComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sdf, grad, rgb, variance, t0, t1, offsets, rays_d, bg, meta):
        n_rays = offsets.numel() - 1
        S = sdf.numel()
        dev = sdf.device
        sdf, grad, rgb = sdf.contiguous(), grad.contiguous(), rgb.contiguous()
        opacity = torch.empty(n_rays, 1, device=dev)
        depth = torch.empty(n_rays, 1, device=dev)
        comp_rgb = torch.empty(n_rays, 3, device=dev)
        comp_normal = torch.empty(n_rays, 3, device=dev)
        comp_full = torch.empty(n_rays, 3, device=dev)
        acc_n = torch.empty(n_rays, 3, device=dev)
        weights = torch.empty(S, device=dev)
        trans = torch.empty(S, device=dev)
        call("angelo_composite_fwd", _p(offsets), n_rays, _p(sdf), _p(grad), _p(t0), _p(t1),
             _p(rays_d), _p(rgb), _p(variance), float(meta["cos_ratio"]), _p(bg),
             float(meta["eps"]), float(meta["gate"]), _p(opacity), _p(depth), _p(comp_rgb),
             _p(comp_normal), _p(comp_full), _p(acc_n), _p(weights), _p(trans),
             _p(meta.get("alpha_out")), _s(dev), units=dict(n=S, rays=n_rays, bwd=False))
        ctx.save_for_backward(sdf, grad, rgb, variance, t0, t1, offsets, rays_d, bg, opacity,
                              acc_n, weights, trans)
        ctx.meta = meta
        ctx.mark_non_differentiable(weights)
        # outputs the loss does not use (opacity, depth, normals) arrive as
        # None, which the kernel reads as zero: no zero-filled gradients
        ctx.set_materialize_grads(False)
        return opacity, depth, comp_rgb, comp_normal, comp_full, weights

    @staticmethod
    def backward(ctx, g_op, g_depth, g_rgb, g_normal, g_full, g_weights):
        (sdf, grad, rgb, variance, t0, t1, offsets, rays_d, bg, opacity, acc_n, weights,
         trans) = ctx.saved_tensors
        meta = ctx.meta
        n_rays = offsets.numel() - 1
        S = sdf.numel()
        dev = sdf.device

        def c(t):
            return t.contiguous().float() if t is not None else None
        d_sdf = torch.empty_like(sdf)
        d_grad = torch.empty_like(grad)
        d_rgb = torch.empty_like(rgb)
        d_var = torch.zeros(1, device=dev)
        call("angelo_composite_bwd", _p(offsets), n_rays, _p(sdf), _p(grad), _p(t0), _p(t1),
             _p(rays_d), _p(rgb), _p(variance), float(meta["cos_ratio"]), _p(bg),
             float(meta["eps"]), float(meta["gate"]), _p(opacity), _p(acc_n), _p(weights),
             _p(trans), _p(c(g_op)), _p(c(g_depth)), _p(c(g_rgb)), _p(c(g_normal)),
             _p(c(g_full)), _p(d_sdf), _p(d_grad), _p(d_rgb), _p(d_var), _s(dev),
             units=dict(n=S, rays=n_rays, bwd=True))
        return (d_sdf, d_grad, d_rgb, d_var.view(variance.shape), None, None, None, None, None,
                None)


def neus_forward(model, rays_o, rays_d, ri, t0, t1, offsets, n_rays, bg_samples=None):
    """NeuSModel.forward_ (models/neus.py:205-283) on the fused kernels:
    fused VolumeSDF -> fused radiance (VolumeRadiance / VolumeDualColor) ->
    fused compositing; VolumeDualColorV3 runs its own module between them."""
    positions, mid = sample_points(rays_o, rays_d, ri, t0, t1)
    sdf, sdf_grad, feature, sdf_laplace = model.geometry(positions, with_grad=True,
                                                         with_feature=True, with_laplace=True)
    ray_indices = ri.long()
    tex = model.texture
    if not FUSED_RENDER:
        return _plain_render(model, rays_o, rays_d, ray_indices, t0, t1, offsets, sdf, sdf_grad,
                             feature, sdf_laplace, bg_samples)
    if type(tex).__name__ in ("VolumeRadiance", "VolumeDualColor") and \
            tex.config.get("color_activation") == "sigmoid":
        rgb = radiance_forward(tex, feature, sdf_grad, ri, rays_d)
    else:
        normal = torch.nn.functional.normalize(sdf_grad, p=2, dim=-1)
        rgb = tex(feature, rays_d[ray_indices], normal)
    bg = model.background_color
    if bg is None:
        raise RuntimeError("set model.background_color before rendering")
    meta = dict(cos_ratio=model.cos_anneal_ratio, eps=1e-4, gate=FP64_ALPHA_GATE)
    variance = model.variance.variance.view(1)
    opacity, depth, comp_rgb, comp_normal, comp_full, weights = _FusedComposite.apply(
        sdf, sdf_grad, rgb, variance, t0, t1, offsets, rays_d, bg.float().contiguous(), meta)
    out = {
        "comp_rgb": comp_rgb, "comp_normal": comp_normal, "opacity": opacity, "depth": depth,
        "rays_valid": opacity > 0,
        "num_samples": torch.full((1,), len(t0), dtype=torch.int32, device=rays_o.device),
    }
    if model.training:
        out.update({"sdf_samples": sdf, "sdf_grad_samples": sdf_grad, "weights": weights,
                    "points": mid, "intervals": t1 - t0, "ray_indices": ray_indices,
                    "sdf_laplace_samples": sdf_laplace})
    out_bg = model.background(out, comp_rgb, rays_o, rays_d, bg_samples)
    if model.learned_background:
        comp_full = comp_rgb + out_bg["comp_rgb"] * (1.0 - opacity)
    out_full = {"comp_rgb": comp_full,
                "num_samples": out["num_samples"] + out_bg["num_samples"],
                "rays_valid": out["rays_valid"] | out_bg["rays_valid"]}
    return {**out, **{k + "_bg": v for k, v in out_bg.items()},
            **{k + "_full": v for k, v in out_full.items()}}


def _plain_render(model, rays_o, rays_d, ray_indices, t0, t1, offsets, sdf, sdf_grad, feature,
                  sdf_laplace, bg_samples=None):
    """The reference's texture / alpha / compositing steps on the library's
    plain kernels, after the fused geometry."""
    from . import ops
    F = torch.nn.functional
    t_dirs = rays_d[ray_indices]
    mid = ((t0 + t1) / 2.0)[:, None]
    dists = (t1 - t0)[:, None]
    normal = F.normalize(sdf_grad, p=2, dim=-1)
    alpha = model.get_alpha(sdf, normal, t_dirs, dists)[..., None]
    rgb = model.texture(feature, t_dirs, normal)
    weights = ops.render_weight_from_alpha(alpha, offsets)[:, None]
    opacity = ops.accumulate_along_rays(weights, offsets)
    depth = ops.accumulate_along_rays(weights, offsets, mid)
    comp_rgb = ops.accumulate_along_rays(weights, offsets, rgb)
    rays_fg = opacity > 0.1
    comp_normal = F.normalize(ops.accumulate_along_rays(weights, offsets, normal), p=2, dim=-1)
    comp_normal = torch.where(rays_fg, comp_normal, torch.zeros_like(comp_normal))
    out = {"comp_rgb": comp_rgb, "comp_normal": comp_normal, "opacity": opacity, "depth": depth,
           "rays_valid": opacity > 0,
           "num_samples": torch.full((1,), len(t0), dtype=torch.int32, device=rays_o.device)}
    if model.training:
        out.update({"sdf_samples": sdf, "sdf_grad_samples": sdf_grad,
                    "weights": weights.view(-1), "points": mid.view(-1),
                    "intervals": dists.view(-1), "ray_indices": ray_indices.view(-1),
                    "sdf_laplace_samples": sdf_laplace})
    return model._with_background(out, comp_rgb, rays_o, rays_d, bg_samples)
