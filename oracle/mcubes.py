"""CPU restatement of the marching-cubes triangulation (test infrastructure
only; the oracle).  The reference triangulates the SDF lattice with PyMCubes
(models/geometry.py:79-113), which is absent here and has no golden vectors in
the reference: parity on the triangulation is unpinned.  This restates the
rule the library documents (include/angelo_gb.h, angelo_mc_*) independently of
its table code: vertices on lattice edges that straddle the level, in edge
order (3 * point + axis), float32 interpolation; per cube the face-walk loops
(iso-lines cut off the corners at or above the level; on each face an
iso-line runs from the edge where the counter-clockwise walk about the
outward normal leaves such a run to the edge where it entered it), each loop
a fan from its smallest-id starting edge."""
from __future__ import annotations

import itertools

import numpy as np


def _corner(c):
    return np.array([c & 1, (c >> 1) & 1, (c >> 2) & 1])


def _edges():
    out = []
    for a in range(3):
        others = [d for d in range(3) if d != a]
        for k in range(4):
            lo = [0, 0, 0]
            lo[others[0]] = k & 1
            lo[others[1]] = (k >> 1) & 1
            hi = list(lo)
            hi[a] = 1
            out.append((lo[0] | lo[1] << 1 | lo[2] << 2, hi[0] | hi[1] << 1 | hi[2] << 2))
    return out


EDGES = _edges()


def _faces():
    faces = []
    for a in range(3):
        for side in range(2):
            cs = [c for c in range(8) if _corner(c)[a] == side]
            n = np.zeros(3)
            n[a] = 1 if side else -1
            ctr = np.mean([_corner(c) for c in cs], 0)
            u = np.zeros(3)
            u[(a + 1) % 3] = 1
            v = np.cross(n, u)
            ang = [np.arctan2(np.dot(_corner(c) - ctr, v), np.dot(_corner(c) - ctr, u)) for c in cs]
            faces.append([cs[i] for i in np.argsort(ang)])
    return faces


FACES = _faces()


def _edge_id(c0, c1):
    for i, (a, b) in enumerate(EDGES):
        if {a, b} == {c0, c1}:
            return i
    raise KeyError((c0, c1))


def cube_triangles(case):
    """Triangles (local edge ids) of a cube whose corner c is at or above the
    level when bit c of `case` is set."""
    pos = [(case >> c) & 1 for c in range(8)]
    nxt = {}
    for q in FACES:
        exits, entries = [], []
        for k in range(4):
            a, b = q[k], q[(k + 1) % 4]
            if pos[a] != pos[b]:
                (exits if pos[a] else entries).append((k, _edge_id(a, b)))
        for k, e in exits:
            before = [x for x in entries if x[0] < k]
            prev = max(before if before else entries, key=lambda x: x[0])
            nxt[e] = prev[1]
    tris, seen = [], set()
    for s in sorted(nxt):
        if s in seen:
            continue
        loop = [s]
        seen.add(s)
        n = nxt[s]
        while n != s:
            loop.append(n)
            seen.add(n)
            n = nxt[n]
        tris += [(loop[0], loop[i], loop[i + 1]) for i in range(1, len(loop) - 1)]
    return tris


TABLE = [cube_triangles(c) for c in range(256)]


def marching_cubes(grid, level, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0)):
    """(vertices float32 (V,3), faces int64 (F,3)) of a float32 lattice."""
    g = np.ascontiguousarray(grid, np.float32)
    nx, ny, nz = g.shape
    lv = np.float32(level)
    o = np.asarray(origin, np.float32)
    sp = np.asarray(spacing, np.float32)
    above = g >= lv
    vid = {}
    verts = []
    for i, j, k in itertools.product(range(nx), range(ny), range(nz)):
        for a in range(3):
            p1 = [i, j, k]
            p1[a] += 1
            if p1[a] >= g.shape[a] or above[i, j, k] == above[tuple(p1)]:
                continue
            v0, v1 = g[i, j, k], g[tuple(p1)]
            t = np.float32(np.float32(lv - v0) / np.float32(v1 - v0))
            q = np.array([i, j, k], np.float32)
            q[a] = np.float32(q[a] + t)
            vid[(i, j, k, a)] = len(verts)
            verts.append(np.float32(o + np.float32(q * sp)))
    faces = []
    for i, j, k in itertools.product(range(nx - 1), range(ny - 1), range(nz - 1)):
        case = 0
        for c in range(8):
            case |= int(above[i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1)]) << c
        for tri in TABLE[case]:
            f = []
            for e in tri:
                c0, c1 = EDGES[e]
                p0 = np.array([i, j, k]) + _corner(c0)
                a = int(np.argmax(_corner(c1) - _corner(c0)))
                f.append(vid[(int(p0[0]), int(p0[1]), int(p0[2]), a)])
            faces.append(f)
    return (np.array(verts, np.float32).reshape(-1, 3), np.array(faces, np.int64).reshape(-1, 3))


# per case: triangle count and the (lower corner, axis) of each triangle edge
_NTRI = np.array([len(t) for t in TABLE], np.int64)
_TRI = np.zeros((256, 5, 3), np.int64)
for _c, _tris in enumerate(TABLE):
    for _t, _tri in enumerate(_tris):
        _TRI[_c, _t] = _tri
_EDGE_LO = np.array([_corner(c0) for c0, _ in EDGES], np.int64)           # (12, 3)
_EDGE_AXIS = np.array([int(np.argmax(_corner(c1) - _corner(c0))) for c0, c1 in EDGES], np.int64)


def marching_cubes_vec(grid, level, origin=(0.0, 0.0, 0.0), spacing=(1.0, 1.0, 1.0)):
    """The same mesh as marching_cubes with whole-array numpy operations (the
    CPU baseline's form; the loop form above is the definition it is tested
    against): vertices in edge order (3 * point + axis), faces in cube order."""
    g = np.ascontiguousarray(grid, np.float32)
    nx, ny, nz = g.shape
    lv = np.float32(level)
    o = np.asarray(origin, np.float32)
    sp = np.asarray(spacing, np.float32)
    above = g >= lv
    cross = np.zeros((nx, ny, nz, 3), bool)
    cross[:-1, :, :, 0] = above[:-1] != above[1:]
    cross[:, :-1, :, 1] = above[:, :-1] != above[:, 1:]
    cross[:, :, :-1, 2] = above[:, :, :-1] != above[:, :, 1:]
    flat = cross.reshape(-1)
    eid = np.nonzero(flat)[0]
    vid_of = np.cumsum(flat, dtype=np.int64) - 1
    p, a = eid // 3, eid % 3
    i, j, k = p // (ny * nz), (p // nz) % ny, p % nz
    idx = np.stack([i, j, k], 1)
    idx1 = idx.copy()
    idx1[np.arange(len(a)), a] += 1
    v0 = g[i, j, k]
    v1 = g[idx1[:, 0], idx1[:, 1], idx1[:, 2]]
    t = ((lv - v0).astype(np.float32) / (v1 - v0).astype(np.float32)).astype(np.float32)
    q = idx.astype(np.float32)
    q[np.arange(len(a)), a] = (q[np.arange(len(a)), a] + t).astype(np.float32)
    verts = (o + (q * sp).astype(np.float32)).astype(np.float32)
    case = np.zeros((nx - 1, ny - 1, nz - 1), np.int64)
    for c in range(8):
        dx, dy, dz = c & 1, (c >> 1) & 1, (c >> 2) & 1
        case |= above[dx:nx - 1 + dx, dy:ny - 1 + dy, dz:nz - 1 + dz].astype(np.int64) << c
    case = case.reshape(-1)
    nt = _NTRI[case]
    cubes = np.nonzero(nt)[0]
    reps = nt[cubes]
    cube_of = np.repeat(cubes, reps)
    tri_of = np.arange(len(cube_of)) - np.repeat(np.cumsum(reps) - reps, reps)
    ci, cj, ck = cube_of // ((ny - 1) * (nz - 1)), (cube_of // (nz - 1)) % (ny - 1), cube_of % (nz - 1)
    e = _TRI[case[cube_of], tri_of]                                       # (F, 3) local edges
    lo = _EDGE_LO[e]                                                      # (F, 3, 3)
    pi, pj, pk = ci[:, None] + lo[..., 0], cj[:, None] + lo[..., 1], ck[:, None] + lo[..., 2]
    gid = ((pi * ny + pj) * nz + pk) * 3 + _EDGE_AXIS[e]
    faces = vid_of[gid]
    return verts.reshape(-1, 3), faces.astype(np.int64).reshape(-1, 3)
