"""torch-facing wrappers of the C ABI: shape/device checks, output allocation
through the PyTorch caching allocator, and torch.autograd.Functions whose
backward passes are the library's hand-written backward kernels.

Every function here runs a kernel of libangelo_gb.so on the current CUDA
stream; none has a CPU path."""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import call

_vp = ctypes.c_void_p


def _p(t):
    return _vp(t.data_ptr()) if t is not None else _vp(0)


# the current stream's handle without constructing a torch Stream object (the
# launches of a step follow one another from the host: a few microseconds
# each that the GPU may wait for)
_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)


def _s(device=None):
    if _raw_stream is not None and isinstance(device, torch.device) and device.type == "cuda" \
            and device.index is not None:
        return _vp(_raw_stream(device.index))
    return _vp(torch.cuda.current_stream(device).cuda_stream)


def _cuda(t, name, dtype=torch.float32, dims=None):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the kernels have no CPU path)")
    if t.dtype != dtype:
        raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
    if dims is not None and t.dim() != dims:
        raise ValueError(f"{name} must have {dims} dims, got {tuple(t.shape)}")
    return t.contiguous()


# ------------------------------------------------------------------ hash grid


class HashGridSpec:
    """Layout of a tcnn-style hash grid (tcnn.Encoding(otype=HashGrid) at
    models/network_utils.py:47), computed by the library on the host."""

    def __init__(self, n_levels, n_features_per_level, log2_hashmap_size, base_resolution,
                 per_level_scale):
        self.desc = _lib.HashGridDesc(int(n_levels), int(n_features_per_level),
                                      int(log2_hashmap_size), int(base_resolution),
                                      float(per_level_scale))
        self.layout = _lib.HashGridLayout()
        call("angelo_hashgrid_layout", ctypes.byref(self.desc), ctypes.byref(self.layout))
        self.n_levels = int(n_levels)
        self.n_features = int(n_features_per_level)
        self.n_entries = int(self.layout.offsets[self.n_levels])
        self.n_params = self.n_entries * self.n_features
        self.n_output_dims = self.n_levels * self.n_features

    @property
    def offsets(self):
        return [int(self.layout.offsets[i]) for i in range(self.n_levels + 1)]

    @property
    def resolutions(self):
        return [int(self.layout.resolutions[i]) for i in range(self.n_levels)]

    @property
    def scales(self):
        return [float(self.layout.scales[i]) for i in range(self.n_levels)]


def _table_dtype(table):
    if table.dtype == torch.float32:
        return _lib.DTYPE_F32
    if table.dtype == torch.float16:
        return _lib.DTYPE_F16
    raise ValueError(f"hash table must be float32 or float16, got {table.dtype}")


def hashgrid_encode_raw(x, table, spec: HashGridSpec, active_levels, include_xyz=True, out=None,
                        out_col=0):
    x = _cuda(x, "x", dims=2)
    if not table.is_cuda or table.numel() != spec.n_params:
        raise ValueError(f"table must be a CUDA tensor of {spec.n_params} values")
    n = x.shape[0]
    width = spec.n_output_dims + (3 if include_xyz else 0)
    if out is None:
        out = torch.empty(n, width, device=x.device, dtype=torch.float32)
        out_col = 0
    call("angelo_hashgrid_fwd", ctypes.byref(spec.layout), int(active_levels), _p(x), n,
         _p(table), _table_dtype(table), int(bool(include_xyz)), _p(out), out.stride(0),
         int(out_col), _s(x.device),
         units=dict(n=n, active=int(active_levels), L=spec.n_levels,
                    tbytes=table.element_size(), xyz=bool(include_xyz)))
    return out


class _HashGridEncode(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, table, spec, active_levels, include_xyz):
        x = x.contiguous()
        out = hashgrid_encode_raw(x, table, spec, active_levels, include_xyz)
        ctx.save_for_backward(x, table)
        ctx.spec, ctx.active, ctx.include_xyz = spec, active_levels, include_xyz
        return out

    @staticmethod
    def backward(ctx, dout):
        x, table = ctx.saved_tensors
        spec = ctx.spec
        dout = dout.contiguous().float()
        need_x, need_t = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        dtable = torch.zeros(spec.n_params, device=x.device, dtype=torch.float32) if need_t else None
        dx = torch.empty_like(x) if need_x else None
        if need_x or need_t:
            call("angelo_hashgrid_bwd", ctypes.byref(spec.layout), int(ctx.active), _p(x),
                 x.shape[0], _p(table), _table_dtype(table), int(bool(ctx.include_xyz)),
                 _p(dout), dout.stride(0), 0, _p(dtable), _p(dx), _s(x.device),
                 launches=int(need_t and ctx.active > 0) + int(need_x),
                 units=dict(n=x.shape[0], active=int(ctx.active), L=spec.n_levels,
                            tbytes=table.element_size(), dtable=bool(need_t), dx=bool(need_x)))
        if dtable is not None and table.dtype != torch.float32:
            dtable = dtable.to(table.dtype)
        return dx, dtable, None, None, None


def hashgrid_encode(x, table, spec: HashGridSpec, active_levels=None, include_xyz=True):
    """Differentiable hash-grid encode (w.r.t. the table and, when x requires
    grad, the input points).  x: (N,3) float32 CUDA in [0,1]."""
    act = spec.n_levels if active_levels is None else int(active_levels)
    return _HashGridEncode.apply(x, table, spec, act, include_xyz)


def hashgrid_index(x, spec: HashGridSpec):
    x = _cuda(x, "x", dims=2)
    n = x.shape[0]
    idx = torch.empty(n, spec.n_levels, 8, device=x.device, dtype=torch.int32)
    w = torch.empty(n, spec.n_levels, 8, device=x.device, dtype=torch.float32)
    call("angelo_hashgrid_index", ctypes.byref(spec.layout), _p(x), n, _p(idx), _p(w),
         _s(x.device))
    return idx, w


# ------------------------------------------------------------------------ SH


class _SH4(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dirs, from_unit):
        dirs = _cuda(dirs, "dirs", dims=2).contiguous()
        out = torch.empty(dirs.shape[0], 16, device=dirs.device, dtype=torch.float32)
        call("angelo_sh4_fwd", _p(dirs), dirs.shape[0], int(from_unit), _p(out), 16, 0,
             _s(dirs.device))
        ctx.save_for_backward(dirs)
        ctx.from_unit = from_unit
        return out

    @staticmethod
    def backward(ctx, dout):
        (dirs,) = ctx.saved_tensors
        if not ctx.needs_input_grad[0]:
            return None, None
        dout = dout.contiguous().float()
        dd = torch.empty_like(dirs)
        call("angelo_sh4_bwd", _p(dirs), dirs.shape[0], int(ctx.from_unit), _p(dout), 16, 0,
             _p(dd), _s(dirs.device))
        return dd, None


def sh4_encode(dirs01):
    """tcnn SphericalHarmonics degree 4 of directions given in [0,1]^3."""
    return _SH4.apply(dirs01, 0)


# ------------------------------------------------------------- ray marching


def ray_aabb_intersect(rays_o, rays_d, aabb):
    rays_o = _cuda(rays_o, "rays_o", dims=2)
    rays_d = _cuda(rays_d, "rays_d", dims=2)
    aabb = _cuda(aabb, "aabb").reshape(6)
    n = rays_o.shape[0]
    t_min = torch.empty(n, device=rays_o.device)
    t_max = torch.empty(n, device=rays_o.device)
    call("angelo_ray_aabb", _p(rays_o), _p(rays_d), n, _p(aabb), _p(t_min), _p(t_max),
         _s(rays_o.device))
    return t_min, t_max


def make_grid_desc(roi, res, bits, contraction=_lib.CONTRACT_AABB):
    g = _lib.GridDesc()
    for i in range(6):
        g.roi[i] = float(roi[i])
    for i in range(3):
        g.res[i] = int(res[i])
    g.bits = bits.data_ptr() if bits is not None else None
    g.contraction = int(contraction)
    return g


UNBOUNDED_ROI = (-1e10, -1e10, -1e10, 1e10, 1e10, 1e10)


MARCH_SCRATCH_BYTES = 1 << 28   # single-march path while its scratch stays below this


def march(rays_o, rays_d, t_min, t_max, step, roi=UNBOUNDED_ROI, res=(1, 1, 1), bits=None,
          cone_angle=0.0, max_steps=1 << 20, max_samples_per_ray=None,
          contraction=_lib.CONTRACT_AABB, before_read=None):
    """Occupancy-grid ray marching.  Returns (ray_indices int32 (S,),
    t_starts (S,), t_ends (S,), offsets int64 (R+1,), status): the sample
    count is read back to the host to size the outputs, as the reference
    does; status is a device int32 tensor (bit 0: a ray reached max_steps)
    that is not read here, so the caller's stream keeps running.

    With max_samples_per_ray (a bound on every ray's sample count, e.g.
    ceil(ray length / step) + 2) each ray is marched once: its samples are
    recorded in a scratch buffer while counting and compacted after the scan;
    a ray over the bound falls back to the second march (same samples).

    before_read: a callable run after the count's copy to the host is
    enqueued and before the host waits for it: work it enqueues (that does
    not depend on the samples) runs on the GPU while the host sizes the
    outputs."""
    rays_o = _cuda(rays_o, "rays_o", dims=2)
    rays_d = _cuda(rays_d, "rays_d", dims=2)
    t_min = _cuda(t_min, "t_min").reshape(-1)
    t_max = _cuda(t_max, "t_max").reshape(-1)
    if bits is not None:
        bits = _cuda(bits, "bits", dtype=torch.int32)
    dev = rays_o.device
    n = rays_o.shape[0]
    g = make_grid_desc(roi, res, bits, contraction)
    counts = torch.empty(n, device=dev, dtype=torch.int32)
    status = torch.zeros(1, device=dev, dtype=torch.int32)
    offsets = torch.empty(n + 1, device=dev, dtype=torch.int64)
    ws = torch.empty(_lib.raw("angelo_scan_workspace_size")(n), device=dev, dtype=torch.uint8)
    s = _s(dev)
    per_ray = int(max_samples_per_ray) if max_samples_per_ray else 0
    single = 0 < per_ray and n * per_ray * 8 <= MARCH_SCRATCH_BYTES
    if single:
        scratch = torch.empty(n * per_ray * 2, device=dev)
        call("angelo_march_record", _p(rays_o), _p(rays_d), _p(t_min), _p(t_max), n,
             ctypes.byref(g), float(step), float(cone_angle), int(max_steps), per_ray,
             _p(scratch), _p(counts), _p(status), s)
    else:
        call("angelo_march_count", _p(rays_o), _p(rays_d), _p(t_min), _p(t_max), n,
             ctypes.byref(g), float(step), float(cone_angle), int(max_steps), _p(counts),
             _p(status), s)
    call("angelo_scan", _p(counts), n, _p(offsets), _p(ws), s, launches=3 if n else 0)
    # the total (and, single-march, the record-overflow bit) in one device read
    head = torch.cat([offsets[n:], status.to(torch.int64)]) if single else offsets[n:]
    if before_read is None:
        vals = head.tolist()
    else:
        host = torch.empty(head.numel(), dtype=torch.int64, pin_memory=True)
        host.copy_(head, non_blocking=True)
        copied = torch.cuda.Event()
        copied.record()
        before_read()
        copied.synchronize()
        vals = host.tolist()
    total = vals[0]
    overflow = single and bool(vals[1] & 4)
    ri = torch.empty(total, device=dev, dtype=torch.int32)
    t0 = torch.empty(total, device=dev)
    t1 = torch.empty(total, device=dev)
    if single and not overflow:
        call("angelo_march_compact", _p(scratch), per_ray, _p(counts), _p(offsets), n, total,
             _p(ri), _p(t0), _p(t1), _p(status), s)
    else:
        call("angelo_march_fill", _p(rays_o), _p(rays_d), _p(t_min), _p(t_max), n,
             ctypes.byref(g), float(step), float(cone_angle), int(max_steps), _p(offsets), total,
             _p(ri), _p(t0), _p(t1), _p(status), s)
    # the outputs are sized by the count pass, so the fill cannot exceed them
    return ri, t0, t1, offsets, status[0]


def scan(counts):
    counts = _cuda(counts, "counts", dtype=torch.int32).reshape(-1)
    n = counts.numel()
    offsets = torch.empty(n + 1, device=counts.device, dtype=torch.int64)
    ws = torch.empty(_lib.raw("angelo_scan_workspace_size")(n), device=counts.device,
                     dtype=torch.uint8)
    call("angelo_scan", _p(counts), n, _p(offsets), _p(ws), _s(counts.device),
         launches=3 if n else 0)
    return offsets


def occ_update(occs, cells, occ, decay, thre, bits):
    """EMA update of the occupancy values (in place) and the bitfield (in place)."""
    occs = _cuda(occs, "occs")
    cells = _cuda(cells, "cells", dtype=torch.int64).reshape(-1)
    occ = _cuda(occ, "occ").reshape(-1)
    bits = _cuda(bits, "bits", dtype=torch.int32)
    n_cells = occs.numel()
    ws = torch.empty(_lib.raw("angelo_occ_workspace_size")(n_cells), device=occs.device,
                     dtype=torch.uint8)
    call("angelo_occ_update", _p(occs), n_cells, _p(cells), _p(occ), cells.numel(), float(decay),
         float(thre), _p(bits), _p(ws), _s(occs.device), launches=5 if cells.numel() else 4)


# ---------------------------------------------------------------- compositing


class _WeightsFromAlpha(torch.autograd.Function):
    @staticmethod
    def forward(ctx, alpha, offsets, early_stop_eps):
        ctx.in_shape = alpha.shape
        alpha = _cuda(alpha, "alpha").reshape(-1)
        offsets = _cuda(offsets, "offsets", dtype=torch.int64)
        n_rays = offsets.numel() - 1
        w = torch.empty_like(alpha)
        trans = torch.empty_like(alpha)
        call("angelo_weights_fwd", _p(alpha), _p(offsets), n_rays, float(early_stop_eps), _p(w),
             _p(trans), _s(alpha.device))
        ctx.save_for_backward(alpha, trans, offsets)
        ctx.eps = early_stop_eps
        return w

    @staticmethod
    def backward(ctx, dw):
        alpha, trans, offsets = ctx.saved_tensors
        dw = dw.contiguous().float().reshape(-1)
        da = torch.empty_like(alpha)
        call("angelo_weights_bwd", _p(alpha), _p(trans), _p(offsets), offsets.numel() - 1,
             float(ctx.eps), _p(dw), _p(da), _s(alpha.device))
        return da.view(ctx.in_shape), None, None


def render_weight_from_alpha(alpha, offsets, early_stop_eps=1e-4):
    return _WeightsFromAlpha.apply(alpha, offsets, early_stop_eps)


@torch.no_grad()
def transmittance_from_alpha(alpha, offsets):
    """T_j = prod_{k<j} (1 - alpha_k) per ray (held once below 1e-4, where
    every later sample is invisible anyway): nerfacc's
    render_transmittance_from_alpha as used by its visibility test."""
    alpha = _cuda(alpha, "alpha").reshape(-1)
    offsets = _cuda(offsets, "offsets", dtype=torch.int64)
    w = torch.empty_like(alpha)
    trans = torch.empty_like(alpha)
    call("angelo_weights_fwd", _p(alpha), _p(offsets), offsets.numel() - 1, 1e-4, _p(w), _p(trans),
         _s(alpha.device))
    return trans


def offsets_from_ray_indices(ray_indices, n_rays):
    """int64 offsets (n_rays + 1) of packed samples sorted by ray."""
    counts = torch.bincount(ray_indices.long(), minlength=n_rays)
    return torch.cat([counts.new_zeros(1), torch.cumsum(counts, 0)])


class _WeightsFromDensity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, t_starts, t_ends, sigmas, offsets):
        ctx.in_shape = sigmas.shape
        t0 = _cuda(t_starts, "t_starts").reshape(-1)
        t1 = _cuda(t_ends, "t_ends").reshape(-1)
        sg = _cuda(sigmas, "sigmas").reshape(-1)
        offsets = _cuda(offsets, "offsets", dtype=torch.int64)
        w = torch.empty_like(sg)
        call("angelo_density_weights_fwd", _p(t0), _p(t1), _p(sg), _p(offsets), offsets.numel() - 1,
             _p(w), _s(sg.device))
        ctx.save_for_backward(t0, t1, sg, w, offsets)
        return w.view(ctx.in_shape)

    @staticmethod
    def backward(ctx, dw):
        t0, t1, sg, w, offsets = ctx.saved_tensors
        dw = dw.contiguous().float().reshape(-1)
        ds = torch.empty_like(sg)
        call("angelo_density_weights_bwd", _p(t0), _p(t1), _p(sg), _p(w), _p(offsets),
             offsets.numel() - 1, _p(dw), _p(ds), _s(sg.device))
        return None, None, ds.view(ctx.in_shape), None


def render_weight_from_density(t_starts, t_ends, sigmas, offsets):
    """nerfacc.render_weight_from_density (models/neus.py:171) over packed
    samples with int64 ray offsets; differentiable in sigmas."""
    return _WeightsFromDensity.apply(t_starts, t_ends, sigmas, offsets)


class _Accumulate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, weights, values, offsets):
        ctx.in_shape = weights.shape
        weights = _cuda(weights, "weights").reshape(-1)
        offsets = _cuda(offsets, "offsets", dtype=torch.int64)
        n_rays = offsets.numel() - 1
        C = 1 if values is None else values.shape[-1]
        if values is not None:
            values = _cuda(values, "values", dims=2)
        out = torch.empty(n_rays, C, device=weights.device)
        call("angelo_accumulate_fwd", _p(weights), _p(values), C, _p(offsets), n_rays, _p(out),
             _s(weights.device))
        ctx.save_for_backward(weights, values, offsets)
        ctx.C = C
        return out

    @staticmethod
    def backward(ctx, dout):
        weights, values, offsets = ctx.saved_tensors
        dout = dout.contiguous().float()
        dw = torch.empty_like(weights)
        dv = torch.empty_like(values) if (values is not None and ctx.needs_input_grad[1]) else None
        call("angelo_accumulate_bwd", _p(weights), _p(values), ctx.C, _p(offsets),
             offsets.numel() - 1, _p(dout), _p(dw), _p(dv), _s(weights.device))
        return dw.view(ctx.in_shape), dv, None


def accumulate_along_rays(weights, offsets, values=None):
    return _Accumulate.apply(weights, values, offsets)
