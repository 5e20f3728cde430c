"""numpy wrappers around the C restatement in ``oracle.c``.

Test infrastructure only: imported by ``tests/``, ``__graft_entry__.smoke`` and
the CPU-baseline leg of ``bench.py`` as the checker.  The product package never
imports this module.

Each wrapper cites the reference call site whose third-party arithmetic it
restates (tcnn HashGrid / SphericalHarmonics, nerfacc 0.3.3).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build() -> str:
    """Compile ``oracle.c`` with its Makefile (idempotent)."""
    src = os.path.join(_HERE, "oracle.c")
    if not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_SO)
            L.or_hashgrid_layout.restype = ctypes.c_uint32
            L.or_hashgrid_layout.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                             _u32p, _u32p, _f32p]
            L.or_hashgrid_index.restype = None
            L.or_hashgrid_index.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, _u32p, _u32p, _f32p,
                                            _u32p, _f32p, _i32p]
            L.or_hashgrid_encode.restype = None
            L.or_hashgrid_encode.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _u32p,
                                             _u32p, _f32p, _f32p, ctypes.c_int, _f32p, ctypes.c_int64]
            L.or_sh4.restype = None
            L.or_sh4.argtypes = [_f32p, ctypes.c_int64, _f64p]
            L.or_ray_aabb.restype = None
            L.or_ray_aabb.argtypes = [_f32p, _f32p, ctypes.c_int64, _f32p, _f32p, _f32p]
            L.or_march.restype = None
            L.or_march.argtypes = [_f32p, _f32p, _f32p, _f32p, ctypes.c_int64, _f32p, _u8p,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                   ctypes.c_float, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
            L.or_weights.restype = None
            L.or_weights.argtypes = [_f32p, _i64p, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                     _f32p, _f32p]
            L.or_occ_binary.restype = None
            L.or_occ_binary.argtypes = [_f32p, ctypes.c_int64, ctypes.c_float, _u32p]
            _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def hashgrid_layout(n_levels, log2_hashmap_size, base_resolution, per_level_scale):
    """Per-level offsets (L+1), resolutions (L) and float32 scales (L) of the
    tcnn hash grid built at models/network_utils.py:47."""
    off = np.zeros(n_levels + 1, np.uint32)
    res = np.zeros(n_levels, np.uint32)
    sc = np.zeros(n_levels, np.float32)
    lib().or_hashgrid_layout(n_levels, log2_hashmap_size, base_resolution, float(per_level_scale),
                             off, res, sc)
    return off, res, sc


def hashgrid_index(x, layout, with_cells=False):
    """Corner entry indices [n, L, 8] (uint32) and weights [n, L, 8] (float32);
    with_cells adds the floor cell of every level [n, L, 3] (int32)."""
    off, res, sc = layout
    x = _c(x, np.float32).reshape(-1, 3)
    n, L = x.shape[0], len(res)
    idx = np.zeros((n, L, 8), np.uint32)
    w = np.zeros((n, L, 8), np.float32)
    cells = np.zeros((n, L, 3), np.int32)
    lib().or_hashgrid_index(x, n, L, off, res, sc, idx, w, cells)
    return (idx, w, cells) if with_cells else (idx, w)


def hashgrid_encode(x, table, layout, n_feat=2, active_levels=None):
    """float32 encode (tcnn HashGrid forward, fp32 params) of x in [0,1]^3."""
    off, res, sc = layout
    x = _c(x, np.float32).reshape(-1, 3)
    n, L = x.shape[0], len(res)
    table = _c(table, np.float32).reshape(-1)
    assert table.size == int(off[-1]) * n_feat
    out = np.zeros((n, L * n_feat), np.float32)
    lib().or_hashgrid_encode(x, n, L, n_feat, off, res, sc, table,
                             L if active_levels is None else int(active_levels), out, L * n_feat)
    return out


def sh4(dirs01):
    """Degree-4 real SH of directions given in [0,1] (models/texture.py:24-25)."""
    d = _c(dirs01, np.float32).reshape(-1, 3)
    out = np.zeros((d.shape[0], 16), np.float64)
    lib().or_sh4(d, d.shape[0], out)
    return out


def ray_aabb(rays_o, rays_d, aabb):
    """nerfacc.intersection.ray_aabb_intersect (models/neus.py:12,153)."""
    o = _c(rays_o, np.float32).reshape(-1, 3)
    d = _c(rays_d, np.float32).reshape(-1, 3)
    n = o.shape[0]
    tmin = np.zeros(n, np.float32)
    tmax = np.zeros(n, np.float32)
    lib().or_ray_aabb(o, d, n, _c(aabb, np.float32), tmin, tmax)
    return tmin, tmax


def march(rays_o, rays_d, t_min, t_max, roi, binary, step, cone=0.0, max_steps=1 << 20,
          contraction=0):
    """nerfacc.ray_marching core (models/neus.py:210-220): returns
    (counts[int32], offsets[int64, n+1], ray_indices[int32], t_starts, t_ends, overflow)."""
    o = _c(rays_o, np.float32).reshape(-1, 3)
    d = _c(rays_d, np.float32).reshape(-1, 3)
    n = o.shape[0]
    tmin = _c(t_min, np.float32).reshape(-1)
    tmax = _c(t_max, np.float32).reshape(-1)
    roi = _c(roi, np.float32).reshape(6)
    b = _c(binary, np.uint8)
    rx, ry, rz = b.shape
    b = b.reshape(-1)
    counts = np.zeros(n, np.int32)
    ovf = np.zeros(1, np.int32)
    L = lib()
    L.or_march(o, d, tmin, tmax, n, roi, b, rx, ry, rz, int(contraction), float(step), float(cone),
               int(max_steps), counts.ctypes.data, None, None, None, None, ovf.ctypes.data)
    offsets = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    tot = int(offsets[-1])
    ri = np.zeros(max(tot, 1), np.int32)
    t0 = np.zeros(max(tot, 1), np.float32)
    t1 = np.zeros(max(tot, 1), np.float32)
    L.or_march(o, d, tmin, tmax, n, roi, b, rx, ry, rz, int(contraction), float(step), float(cone),
               int(max_steps), None, offsets.ctypes.data, ri.ctypes.data, t0.ctypes.data,
               t1.ctypes.data, ovf.ctypes.data)
    return counts, offsets, ri[:tot], t0[:tot], t1[:tot], bool(ovf[0])


def weights(alpha, offsets, early_stop_eps=1e-4, alpha_thre=0.0):
    """nerfacc.render_weight_from_alpha (models/neus.py:234): (weights, transmittance)."""
    a = _c(alpha, np.float32).reshape(-1)
    off = _c(offsets, np.int64)
    w = np.zeros_like(a)
    t = np.zeros_like(a)
    lib().or_weights(a, off, len(off) - 1, float(early_stop_eps), float(alpha_thre), w, t)
    return w, t


def occ_binary(occ, thre):
    """Bitfield of OccupancyGrid._update's threshold step (models/neus.py:109)."""
    occ = _c(occ, np.float32).reshape(-1)
    bits = np.zeros((occ.size + 31) // 32, np.uint32)
    lib().or_occ_binary(occ, occ.size, float(thre), bits)
    return bits
