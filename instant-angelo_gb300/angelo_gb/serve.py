"""Serving loop for a trained NeuS field: novel-view renders and SDF query
lattices (the marching-cubes grids of VolumeSDF.isosurface).

The trained state (hash table, MLP weights, occupancy bitfield) stays resident
on the device.  Requests of uneven size arrive over time; the loop admits them
while enough HBM is free, cuts them into fixed-shape buckets (rays or lattice
points) and runs the buckets of all admitted requests back to back as
CUDA-graph replays on two streams, so renders and SDF grids overlap on the
device (two render buckets take turns, so renders also overlap each other).
Completion is observed through events: a request that arrives while others
are on the GPU joins the next bucket.

A render bucket is: clip to the near/far planes or the scene box, march
(count, scan, fill into a fixed sample capacity), the fused VolumeSDF (the
point and its 6 FD taps: the normal needs them, the curvature does not), the
fused radiance network and the fused compositing.  Nothing in it synchronises
with the host, so it is captured once.  A bucket whose samples overflow the
capacity is re-rendered through the exact-size path (the same kernels); its
offsets are clamped to the capacity first, so the bucket's own compositing
reads and writes only the samples the fill kept.

The reference serves one request at a time through NeuSModel.forward in eval
mode, in 2048-ray chunks moved to the CPU (models/neus.py:285-293,
models/utils.py:14-51); ``sequential_plain`` measures that path.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import time
from collections import deque

import numpy as np
import torch

from . import _lib, fused, ops, scenes


@dataclasses.dataclass
class RenderRequest:
    rid: int
    c2w: torch.Tensor          # (3, 4) camera-to-world
    W: int
    H: int
    fov: float = 40.0
    arrival: float = 0.0       # seconds after the loop starts
    rgb: torch.Tensor = None   # (H*W, 3) result, background blended
    opacity: torch.Tensor = None
    depth: torch.Tensor = None
    done: float = None         # completion time, seconds after the start
    next_ray: int = 0
    pending: int = 0

    @property
    def n(self):
        return self.W * self.H


@dataclasses.dataclass
class SdfGridRequest:
    rid: int
    res: int                   # lattice points per axis over [-r, r]
    arrival: float = 0.0
    sdf: torch.Tensor = None   # (res^3,) result, x-major
    done: float = None
    next_pt: int = 0
    pending: int = 0

    @property
    def n(self):
        return self.res ** 3


def request_rays(req: RenderRequest, start, n, device):
    """Rays [start, start + n) of a render request (row-major pixels,
    pinhole camera looking down -z)."""
    f = req.W / (2 * math.tan(math.radians(req.fov) / 2))
    idx = torch.arange(start, start + n, device=device)
    i = (idx % req.W).float() + 0.5
    j = torch.div(idx, req.W, rounding_mode="floor").float() + 0.5
    dirs = torch.stack([(i - req.W / 2) / f, -(j - req.H / 2) / f, -torch.ones_like(i)], -1)
    c2w = req.c2w.to(device=device, dtype=torch.float32)
    return scenes.rays_from(dirs, c2w[None].expand(n, 3, 4))


def request_points(req: SdfGridRequest, start, n, radius, device):
    """Lattice points [start, start + n) of a res^3 grid over [-r, r]^3
    (x-major, the point order of VolumeSDF.isosurface's helper)."""
    idx = torch.arange(start, start + n, device=device)
    r = req.res
    ix = torch.div(idx, r * r, rounding_mode="floor")
    iy = torch.div(idx, r, rounding_mode="floor") % r
    iz = idx % r
    step = 2.0 * radius / (r - 1)
    return torch.stack([ix, iy, iz], -1).float() * step - radius


def _t_range(model, o, d):
    """Near/far planes or the scene box, as NeuSModel.march_rays without the
    training jitter."""
    if model.near_plane is None and model.far_plane is None:
        return ops.ray_aabb_intersect(o, d, model.scene_aabb)
    t_min = torch.zeros_like(o[:, 0])
    t_max = torch.full_like(o[:, 0], 1e10)
    if model.near_plane is not None:
        t_min = t_min.clamp(min=model.near_plane)
    if model.far_plane is not None:
        t_max = t_max.clamp(max=model.far_plane)
    return t_min, t_max


def _grid_desc(model):
    if model.config.grid_prune:
        g = model.occupancy_grid
        return ops.make_grid_desc(g.roi, (g.res,) * 3, g.bits)
    return ops.make_grid_desc(ops.UNBOUNDED_ROI, (1, 1, 1), None)


def _shade(model, o, d, ri, t0, t1, offsets, bg):
    """Fused geometry (point + FD taps) -> fused radiance -> fused compositing
    of packed samples; returns (rgb with background, opacity, depth)."""
    ray_indices = ri.long()
    mid = (t0 + t1) * 0.5
    pos = o[ray_indices] + d[ray_indices] * mid[:, None]
    sdf, grad, feat = fused.volume_sdf_forward(model.geometry, pos, True, True, False)
    rgb = fused.radiance_forward(model.texture, feat, grad, ri, d)
    meta = dict(cos_ratio=1.0, eps=1e-4, gate=fused.FP64_ALPHA_GATE)
    var = model.variance.variance.view(1)
    op, dep, comp, cn, full, w = fused._FusedComposite.apply(sdf, grad, rgb, var, t0, t1, offsets, d,
                                                             bg, meta)
    return full, op, dep


@torch.no_grad()
def render_exact(model, rays, bg):
    """The same render with exact sizes (march with a host read of the sample
    count); the overflow path of a bucket and the reference of the tests."""
    o, d = rays[:, :3].contiguous(), rays[:, 3:].contiguous()
    t_min, t_max = _t_range(model, o, d)
    if model.config.grid_prune:
        g = model.occupancy_grid
        grid = dict(roi=g.roi, res=(g.res,) * 3, bits=g.bits)
    else:
        grid = dict(roi=ops.UNBOUNDED_ROI, res=(1, 1, 1), bits=None)
    ri, t0, t1, offsets, _ = ops.march(o, d, t_min, t_max, model.render_step_size, cone_angle=0.0,
                                       max_steps=model.max_march_steps, **grid)
    return _shade(model, o, d, ri, t0, t1, offsets, bg)


class RenderBucket:
    """Fixed-shape render of up to B rays with a fixed sample capacity,
    captured once as a CUDA graph and replayed."""

    def __init__(self, model, B, max_samples_per_ray, stream, bg, use_graph=True):
        self.m, self.B, self.stream = model, int(B), stream
        self.cap = int(B) * int(max_samples_per_ray)
        dev = model.scene_aabb.device
        z = lambda *s, dt=torch.float32: torch.zeros(*s, device=dev, dtype=dt)  # noqa: E731
        self.rays = z(self.B, 6)
        self.rays[:, 3] = 1.0
        self.counts = z(self.B, dt=torch.int32)
        self.offsets = z(self.B + 1, dt=torch.int64)
        self.scan_ws = z(_lib.raw("angelo_scan_workspace_size")(self.B), dt=torch.uint8)
        self.status = z(1, dt=torch.int32)
        self.ri = z(self.cap, dt=torch.int32)
        self.t0 = z(self.cap)
        self.t1 = z(self.cap) + 1e-3
        self.grid = _grid_desc(model)
        self.bg = bg.float().contiguous()
        self.graph = None
        self.use_graph = use_graph

    def _body(self):
        m = self.m
        o, d = self.rays[:, :3], self.rays[:, 3:]
        oc, dc = o.contiguous(), d.contiguous()
        t_min, t_max = _t_range(m, oc, dc)
        s = ops._s(oc.device)
        P = ops._p
        _lib.call("angelo_march_count", P(oc), P(dc), P(t_min), P(t_max), self.B,
                  ctypes.byref(self.grid), float(m.render_step_size), 0.0, int(m.max_march_steps),
                  P(self.counts), P(self.status), s)
        _lib.call("angelo_scan", P(self.counts), self.B, P(self.offsets), P(self.scan_ws), s)
        _lib.call("angelo_march_fill", P(oc), P(dc), P(t_min), P(t_max), self.B,
                  ctypes.byref(self.grid), float(m.render_step_size), 0.0, int(m.max_march_steps),
                  P(self.offsets), self.cap, P(self.ri), P(self.t0), P(self.t1), P(self.status), s)
        # an overflowing bucket keeps the samples below the capacity: clamp
        # the offsets so the compositing walks only those (the bucket is then
        # re-rendered exactly, status bit 1)
        _lib.call("angelo_offsets_clamp", P(self.offsets), self.B, self.cap, s)
        self.out = _shade(m, oc, dc, self.ri, self.t0, self.t1, self.offsets, self.bg)

    @torch.no_grad()
    def prepare(self):
        with torch.cuda.stream(self.stream):
            self._body()        # warm-up: allocations, kernel attributes
        self.stream.synchronize()
        if self.use_graph:
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=self.stream):
                self._body()
        self.stream.synchronize()

    @torch.no_grad()
    def launch(self, rays, n):
        """Render rays[:n] (n <= B) on the bucket's stream; the returned
        tensors are valid once the stream reaches this point."""
        with torch.cuda.stream(self.stream):
            self.rays[:n].copy_(rays[:n])
            if n < self.B:
                self.rays[n:].zero_()
                self.rays[n:, 3] = 1.0
            self.status.zero_()
            if self.graph is not None:
                self.graph.replay()
            else:
                self._body()
            full, op, dep = self.out
            return full[:n].clone(), op[:n].clone(), dep[:n].clone(), self.status.clone()


class SdfBucket:
    """Fixed-shape SDF query of B lattice points (VolumeSDF.forward_level on
    the fused kernels), graph-captured."""

    def __init__(self, model, B, stream, use_graph=True):
        self.m, self.B, self.stream = model, int(B), stream
        self.pts = torch.zeros(self.B, 3, device=model.scene_aabb.device)
        self.graph = None
        self.use_graph = use_graph

    def _body(self):
        self.out = fused.sdf_query(self.m.geometry, self.pts)

    @torch.no_grad()
    def prepare(self):
        with torch.cuda.stream(self.stream):
            self._body()
        self.stream.synchronize()
        if self.use_graph:
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self.graph, stream=self.stream):
                self._body()
        self.stream.synchronize()

    @torch.no_grad()
    def launch(self, pts, n):
        with torch.cuda.stream(self.stream):
            self.pts[:n].copy_(pts[:n])
            if self.graph is not None:
                self.graph.replay()
            else:
                self._body()
            return self.out[:n].clone()


class NativeServer:
    """The library's own server (angelo_serve_*: C ABI, buckets replayed as a
    CUDA graph) over a NeuSModel's resident state: renders and SDF queries
    with the kernels and order of RenderBucket / SdfBucket.  The weights are
    prepared once; the model must not change while the server lives."""

    def __init__(self, model, rays_per_bucket=1 << 14, samples_per_ray=128,
                 points_per_bucket=1 << 20, background=(1.0, 1.0, 1.0), use_graph=True):
        geom, tex = model.geometry, model.texture
        dev = model.scene_aabb.device
        self.model = model
        self.sdf_net = fused._net_for(geom)
        self.sdf_net.layout.mma_passes = 3
        self.sdf_net.prepare(fused.effective_weights(geom.network))
        od = self.sdf_net.out_dim
        self.rad_net = fused.RadNet(od + 3, dev)
        self.rad_net.prepare(tex.network.effective_weights())
        self.bg = torch.as_tensor(background, dtype=torch.float32, device=dev).contiguous()
        self.var = model.variance.variance.detach().reshape(1).float().contiguous()
        table = geom.hashgrid.encoding.params
        f = _lib.ServeField()
        f.lay = geom.hashgrid.encoding.spec.layout
        f.active_levels = int(geom.hashgrid.mask_levels)
        f.table = table.data_ptr()
        f.table_dtype = _lib.DTYPE_F32 if table.dtype == torch.float32 else _lib.DTYPE_F16
        f.sdf_layout = self.sdf_net.layout
        f.sdf_net = self.sdf_net.buf.data_ptr()
        f.radius = float(geom.radius)
        f.eps = float(geom._finite_difference_eps or 1.0)
        f.feat_dim = od + 3
        f.rad_net = self.rad_net.buf.data_ptr()
        f.rad_flags = int(bool(getattr(tex, "dual", False)))
        f.variance = self.var.data_ptr()
        f.cos_anneal_ratio = 1.0
        f.background = self.bg.data_ptr()
        f.grid = _grid_desc(model)
        f.render_step = float(model.render_step_size)
        f.max_steps = int(min(model.max_march_steps, (1 << 31) - 1))
        f.near_plane = -1.0 if model.near_plane is None else float(model.near_plane)
        f.far_plane = -1.0 if model.far_plane is None else float(model.far_plane)
        self.field = f
        self.handle = ctypes.c_void_p()
        _lib.call("angelo_serve_create", ctypes.byref(f), int(rays_per_bucket), int(samples_per_ray),
                  int(points_per_bucket), int(use_graph), ctypes.byref(self.handle))

    @torch.no_grad()
    def render(self, rays):
        """rays (n, 6) on the device -> (rgb with background, opacity, depth,
        number of buckets rendered again at exact size)."""
        o, d = rays[:, :3].contiguous().float(), rays[:, 3:].contiguous().float()
        n = o.shape[0]
        rgb = torch.empty(n, 3, device=o.device)
        op = torch.empty(n, 1, device=o.device)
        dep = torch.empty(n, 1, device=o.device)
        ovf = ctypes.c_int64(0)
        _lib.call("angelo_serve_render", self.handle, ops._p(o), ops._p(d), n, ops._p(rgb), ops._p(op),
                  ops._p(dep), ctypes.byref(ovf), ops._s(o.device))
        return rgb, op, dep, int(ovf.value)

    @torch.no_grad()
    def sdf(self, points):
        p = points.reshape(-1, 3).contiguous().float()
        out = torch.empty(p.shape[0], device=p.device)
        _lib.call("angelo_serve_sdf", self.handle, ops._p(p), p.shape[0], ops._p(out), ops._s(p.device))
        return out.view(points.shape[:-1])

    def close(self):
        if self.handle:
            _lib.call("angelo_serve_destroy", self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous batching over RenderBucket / SdfBucket replays.

    ray_bucket rays per render bucket (each at most max_samples_per_ray
    samples), point_bucket lattice points per SDF bucket; a request is
    admitted when the HBM left after its result buffers stays above
    hbm_reserve bytes.  render_streams render buckets (each its own captured
    graph, buffers and stream) take turns, so consecutive render buckets
    overlap on the device as well as renders and SDF grids."""

    def __init__(self, model, ray_bucket=1 << 14, max_samples_per_ray=128, point_bucket=1 << 20,
                 use_graph=True, hbm_reserve=4 << 30, background=(1.0, 1.0, 1.0),
                 render_streams=2):
        if not torch.cuda.is_available():
            raise RuntimeError("the serving loop runs on the GPU")
        self.m = model.eval()
        dev = model.scene_aabb.device
        self.dev = dev
        self.bg = torch.tensor(background, device=dev, dtype=torch.float32)
        self.rbs = [RenderBucket(model, ray_bucket, max_samples_per_ray, torch.cuda.Stream(dev),
                                 self.bg, use_graph) for _ in range(max(1, int(render_streams)))]
        self.rb = self.rbs[0]
        self.ss = torch.cuda.Stream(dev)
        self.sb = SdfBucket(model, point_bucket, self.ss, use_graph)
        for rb in self.rbs:
            rb.prepare()
        self.sb.prepare()
        self.reserve = int(hbm_reserve)
        self.overflows = 0
        self.buckets = 0

    def _mem_ok(self, req):
        free, _ = torch.cuda.mem_get_info(self.dev)
        need = req.n * (4 * 5 if isinstance(req, RenderRequest) else 4) + (64 << 20)
        return free - need > self.reserve

    def _finish_render_bucket(self, parts, st, rays):
        """Overflowed sample capacity: re-render the bucket's rays exactly."""
        if int(st.item()) & 2 == 0:
            return
        self.overflows += 1
        full, op, dep = render_exact(self.m, rays, self.bg)
        o = 0
        for q, s, n in parts:
            q.rgb[s:s + n].copy_(full[o:o + n])
            q.opacity[s:s + n].copy_(op[o:o + n])
            q.depth[s:s + n].copy_(dep[o:o + n])
            o += n

    @torch.no_grad()
    def run(self, requests, realtime=True):
        """Serve requests (their .arrival in seconds from the start; with
        realtime=False all are present at once).  Fills each request's
        result and .done, and returns the requests."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        active_r, active_s, inflight = [], [], deque()
        t0 = time.perf_counter()
        done = 0
        turn = 0
        while done < len(requests):
            now = time.perf_counter() - t0
            while pending and (pending[0].arrival <= now or not realtime) and \
                    (self._mem_ok(pending[0]) or not (active_r or active_s or inflight)):
                # (a request is admitted alone when nothing else holds memory)
                q = pending.popleft()
                if isinstance(q, RenderRequest):
                    q.rgb = torch.empty(q.n, 3, device=self.dev)
                    q.opacity = torch.empty(q.n, 1, device=self.dev)
                    q.depth = torch.empty(q.n, 1, device=self.dev)
                    active_r.append(q)
                else:
                    q.sdf = torch.empty(q.n, device=self.dev)
                    active_s.append(q)
            if not active_r and not active_s and not inflight and pending and \
                    pending[0].arrival > now and realtime:
                time.sleep(min(1e-3, pending[0].arrival - now))
                continue
            launched = False
            if active_r:
                # one render bucket, filled from the active renders in turn
                budget, parts, k = self.rb.B, [], 0
                while budget > 0 and k < len(active_r):
                    q = active_r[(turn + k) % len(active_r)]
                    take = min(budget, q.n - q.next_ray)
                    if take > 0:
                        parts.append((q, q.next_ray, take))
                        q.next_ray += take
                        budget -= take
                    k += 1
                turn += 1
                if parts:
                    rb = self.rbs[self.buckets % len(self.rbs)]
                    with torch.cuda.stream(rb.stream):
                        rays = torch.cat([request_rays(q, s, n, self.dev) for q, s, n in parts])
                    full, op, dep, st = rb.launch(rays, rays.shape[0])
                    o = 0
                    with torch.cuda.stream(rb.stream):
                        for q, s, n in parts:
                            q.rgb[s:s + n].copy_(full[o:o + n])
                            q.opacity[s:s + n].copy_(op[o:o + n])
                            q.depth[s:s + n].copy_(dep[o:o + n])
                            o += n
                            q.pending += 1
                        ev = torch.cuda.Event()
                        ev.record(rb.stream)
                    inflight.append((ev, parts, st, rays))
                    self.buckets += 1
                    launched = True
            if active_s:
                q = active_s[0]
                take = min(self.sb.B, q.n - q.next_pt)
                if take > 0:
                    with torch.cuda.stream(self.ss):
                        pts = request_points(q, q.next_pt, take, float(self.m.config.radius), self.dev)
                    sdf = self.sb.launch(pts, take)
                    with torch.cuda.stream(self.ss):
                        q.sdf[q.next_pt:q.next_pt + take].copy_(sdf)
                        ev = torch.cuda.Event()
                        ev.record(self.ss)
                    q.next_pt += take
                    q.pending += 1
                    inflight.append((ev, [(q, 0, 0)], None, None))
                    self.buckets += 1
                    launched = True
            # completions; block on the oldest only when nothing new was launched
            while inflight and (inflight[0][0].query() or not launched):
                ev, parts, st, rays = inflight.popleft()
                ev.synchronize()
                if st is not None:
                    self._finish_render_bucket(parts, st, rays)
                t = time.perf_counter() - t0
                for q, _, _ in parts:
                    q.pending -= 1
                    if isinstance(q, RenderRequest):
                        finished = q.next_ray >= q.n
                    else:
                        finished = q.next_pt >= q.n
                    if finished and q.pending == 0 and q.done is None:
                        q.done = t
                        done += 1
                        (active_r if isinstance(q, RenderRequest) else active_s).remove(q)
                launched = True
        torch.cuda.synchronize(self.dev)
        return requests


def latency_stats(requests):
    """p50 / p99 of completion minus arrival, in milliseconds."""
    lat = np.array([(q.done - q.arrival) * 1e3 for q in requests])
    return float(np.percentile(lat, 50)), float(np.percentile(lat, 99))


@torch.no_grad()
def sequential_plain(model_plain, requests, background=(1.0, 1.0, 1.0)):
    """The reference's serving path: one request at a time, in arrival order,
    through NeuSModel.forward in eval mode (2048-ray chunks moved to the CPU)
    on the plain kernels; SDF grids through forward_level in 2^18-point
    chunks.  Fills .done (a request starts when both it has arrived and the
    previous one finished) and returns the requests."""
    m = model_plain.eval()
    dev = m.scene_aabb.device
    m.background_color = torch.tensor(background, device=dev)
    t0 = time.perf_counter()
    for q in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if q.arrival > now:
            time.sleep(q.arrival - now)
        if isinstance(q, RenderRequest):
            rays = request_rays(q, 0, q.n, dev)
            out = m(rays)
            q.rgb = out["comp_rgb_full"]
        else:
            parts = []
            for s in range(0, q.n, 1 << 18):
                n = min(1 << 18, q.n - s)
                pts = request_points(q, s, n, float(m.config.radius), dev)
                parts.append(m.geometry.forward_level(pts).cpu())
            q.sdf = torch.cat(parts)
        torch.cuda.synchronize(dev)
        q.done = time.perf_counter() - t0
    return requests
