"""Marching cubes on the GPU (libangelo_gb angelo_mc_*), the triangulation
step of MarchingCubeHelper (models/geometry.py:79-113), which the reference
runs through PyMCubes on the host block by block."""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import call
from .ops import _p, _s


def marching_cubes(grid, level, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0)):
    """Isosurface of a float32 (nx, ny, nz) lattice at `level`: returns
    (vertices (V, 3) float32 = origin + index * spacing, faces (F, 3) int64),
    on the lattice's device (a host lattice is moved to the current GPU).
    Vertices are shared between adjacent cubes; triangles face the higher
    values."""
    g = grid
    if not g.is_cuda:
        g = g.to("cuda")
    g = g.float().contiguous()
    if g.dim() != 3 or min(g.shape) < 2:
        raise ValueError(f"marching_cubes: lattice of shape {tuple(g.shape)}")
    nx, ny, nz = (int(v) for v in g.shape)
    dev = g.device
    ws = torch.empty(_lib.raw("angelo_mc_workspace_size")(nx, ny, nz), dtype=torch.uint8, device=dev)
    totals = torch.zeros(2, dtype=torch.int64, device=dev)
    call("angelo_mc_count", _p(g), nx, ny, nz, float(level), _p(ws), _p(totals), _s(dev), launches=8)
    n_v, n_f = (int(v) for v in totals.cpu())
    verts = torch.empty(n_v, 3, device=dev)
    faces = torch.empty(n_f, 3, dtype=torch.int64, device=dev)
    o = (ctypes.c_float * 3)(*[float(v) for v in origin])
    sp = (ctypes.c_float * 3)(*[float(v) for v in spacing])
    call("angelo_mc_extract", _p(g), nx, ny, nz, float(level), o, sp, _p(ws),
         _p(verts) if n_v else None, _p(faces) if n_f else None, _s(dev), launches=2)
    return verts, faces
