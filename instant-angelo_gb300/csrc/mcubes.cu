// Marching cubes on the GPU: the isosurface of an SDF lattice, replacing the
// reference's PyMCubes call on the host (models/geometry.py:79-113, 144-149).
//
// One vertex per lattice edge whose end values straddle the level (value >=
// level on one end only), at the linear interpolation t = (level - v0) /
// (v1 - v0) from the edge's lower end, so that cubes sharing the edge share
// the vertex.  Each cube's triangles come from a 256-case table generated on
// the host by a face-walk rule: on every cube face the iso-lines cut off the
// runs of corners at or above the level (a face with two such corners on a
// diagonal is cut into two), each iso-line runs from the edge where the
// counter-clockwise walk (about the outward normal) leaves the run to the
// edge where it entered it, the lines chain into closed loops across faces,
// and every loop is a triangle fan.  Neighbouring cubes apply the rule to
// their common face, so the mesh is closed wherever the surface does not
// leave the lattice, and triangles face the higher values.
//
// Passes: per 32-point chunk of a lattice row, crossing masks + vertex and
// triangle counts -> scans over chunks -> vertices and faces (vertex ids
// from chunk offsets and mask popcounts).
#include <stdint.h>

#include <mutex>

#include "common.cuh"

using namespace angelo;

namespace {

constexpr int kMaxTri = 5;   // triangles per cube case

// per case: [0] = triangle count, then 3 local edge ids per triangle
__constant__ int8_t c_tri[256][1 + 3 * kMaxTri];

// ---------------------------------------------------------------- the table
// corner c: (x, y, z) = (c & 1, c >> 1 & 1, c >> 2 & 1); edges 0-3 along x,
// 4-7 along y, 8-11 along z (the edge of axis a and index k has the other two
// coordinates (k & 1, k >> 1) in increasing axis order)

struct CubeTopology {
    int edge_c[12][2];   // corners of each edge (lower, upper)
    int face_c[6][4];    // corners of each face, counter-clockwise about the outward normal
};

CubeTopology make_topology() {
    CubeTopology T{};
    for (int a = 0; a < 3; ++a) {
        const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
        for (int k = 0; k < 4; ++k) {
            int lo[3] = {0, 0, 0};
            lo[o0] = k & 1;
            lo[o1] = (k >> 1) & 1;
            int hi[3] = {lo[0], lo[1], lo[2]};
            hi[a] = 1;
            T.edge_c[4 * a + k][0] = lo[0] | lo[1] << 1 | lo[2] << 2;
            T.edge_c[4 * a + k][1] = hi[0] | hi[1] << 1 | hi[2] << 2;
        }
    }
    // face of axis a, side s: the four corners with coordinate a == s in the
    // cyclic order (u, v) = (0,0), (1,0), (1,1), (0,1) of the two other axes
    // (u = a+1, v = a+2 mod 3), which is counter-clockwise about +a; the
    // side-0 face (outward normal -a) takes the reverse order
    int f = 0;
    for (int a = 0; a < 3; ++a) {
        const int u = (a + 1) % 3, v = (a + 2) % 3;
        const int cyc[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        for (int s = 0; s < 2; ++s, ++f) {
            for (int i = 0; i < 4; ++i) {
                const int j = s == 1 ? i : (4 - i) % 4;
                int p[3];
                p[a] = s;
                p[u] = cyc[j][0];
                p[v] = cyc[j][1];
                T.face_c[f][i] = p[0] | p[1] << 1 | p[2] << 2;
            }
        }
    }
    return T;
}

int edge_of(const CubeTopology &T, int c0, int c1) {
    for (int e = 0; e < 12; ++e)
        if ((T.edge_c[e][0] == c0 && T.edge_c[e][1] == c1) || (T.edge_c[e][0] == c1 && T.edge_c[e][1] == c0))
            return e;
    return -1;
}

void make_table(int8_t (*tab)[1 + 3 * kMaxTri]) {
    const CubeTopology T = make_topology();
    for (int cs = 0; cs < 256; ++cs) {
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int f = 0; f < 6; ++f) {
            int ex_k[2], ex_e[2], en_k[2], en_e[2], nex = 0, nen = 0;
            for (int k = 0; k < 4; ++k) {
                const int a = T.face_c[f][k], b = T.face_c[f][(k + 1) % 4];
                const int pa = (cs >> a) & 1, pb = (cs >> b) & 1;
                if (pa == pb) continue;
                if (pa) {
                    ex_k[nex] = k;
                    ex_e[nex++] = edge_of(T, a, b);
                } else {
                    en_k[nen] = k;
                    en_e[nen++] = edge_of(T, a, b);
                }
            }
            // each exit pairs with the previous entry along the walk
            for (int i = 0; i < nex; ++i) {
                int best = -1, best_k = -1;
                for (int j = 0; j < nen; ++j)
                    if (en_k[j] < ex_k[i] && en_k[j] > best_k) best = j, best_k = en_k[j];
                if (best < 0)
                    for (int j = 0; j < nen; ++j)
                        if (en_k[j] > best_k) best = j, best_k = en_k[j];
                next[ex_e[i]] = en_e[best];
            }
        }
        int n_tri = 0;
        bool seen[12] = {};
        int8_t *row = tab[cs];
        for (int s = 0; s < 12; ++s) {
            if (next[s] < 0 || seen[s]) continue;
            int loop[12], n = 0;
            for (int e = s; !seen[e]; e = next[e]) {
                seen[e] = true;
                loop[n++] = e;
            }
            for (int i = 1; i + 1 < n && n_tri < kMaxTri; ++i, ++n_tri) {
                row[1 + 3 * n_tri] = (int8_t)loop[0];
                row[2 + 3 * n_tri] = (int8_t)loop[i];
                row[3 + 3 * n_tri] = (int8_t)loop[i + 1];
            }
        }
        row[0] = (int8_t)n_tri;
    }
}

// upload once per device (the constant bank is per context)
int ensure_table() {
    static std::mutex mu;
    static uint64_t done = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("mcubes(device)");
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && (done >> dev) & 1) return ANGELO_OK;
    static int8_t tab[256][1 + 3 * kMaxTri];
    static bool built = false;
    if (!built) {
        make_table(tab);
        built = true;
    }
    if (cudaMemcpyToSymbol(c_tri, tab, sizeof(tab)) != cudaSuccess) return check_launch("mcubes(table)");
    if (dev < 64) done |= 1ull << dev;
    return ANGELO_OK;
}

// ------------------------------------------------------------------ kernels
//
// Lattice rows: row r = (i, j) = (r / ny, r % ny) holds the points k = 0 ..
// nz - 1 (point index r * nz + k), cut into chunks of 32 points (work item
// r * nw + w, nw = ceil(nz / 32)).  A vertex's id is its edge's rank in the
// order (point, axis), so within a chunk vertices run by k, then axis.  Each
// chunk keeps three crossing bitmasks (one 32-bit word per axis, bit k - 32 w:
// the edge from (i, j, k) along that axis crosses the level); a vertex's id is
// its chunk's offset plus popcounts of the chunk's words below it.  For a
// 512^3 lattice the masks are 50 MB and stay in L2 between the passes.
//
// One warp per work item.  Pass 1 writes the masks and per item the vertex
// count and the triangle count of its cubes (i, j, k) (none for i = nx - 1 or
// j = ny - 1, so that the item order is the cube order).  Pass 2 recomputes
// the item's cube cases and writes its vertices and the faces of its cubes,
// reading the masks and offsets of the four rows a cube touches.

constexpr int kMcWarps = 8;   // warps per block

struct Lattice {
    const float *v;
    int nx, ny, nz;
    float level;
    __device__ __forceinline__ float at(int ii, int jj, int k) const {
        return v[((int64_t)ii * ny + jj) * nz + k];
    }
};

// the four rows a cube row touches: q = dx | dy << 1 -> (i + dx, j + dy)
struct Chunk {
    float v[4];        // this lane's values at k = kb + lane of rows q (0 outside)
    uint32_t up[4];    // ballots: value >= level, bit = lane
    uint32_t next;     // bit q: the value at k = kb + 32 of row q is >= level
    float v_next;      // row 0's value at kb + 32 (lane 31 only)
};

// kMcGroup consecutive chunks of row (i, j) from chunk w0: every load issued
// before the first ballot (the chunks' latencies overlap)
constexpr int kMcGroup = 4;

__device__ __forceinline__ void load_group(const Lattice &L, int i, int j, int w0, int lane, Chunk (&C)[kMcGroup]) {
    float v[kMcGroup][4];
    float vend[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int u = 0; u < kMcGroup; ++u) {
        const int k = 32 * (w0 + u) + lane;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int ii = i + (q & 1), jj = j + (q >> 1);
            v[u][q] = (ii < L.nx && jj < L.ny && k < L.nz) ? L.at(ii, jj, k) : 0.0f;
        }
    }
    const int kend = 32 * (w0 + kMcGroup);
    if (lane == 31 && kend < L.nz) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int ii = i + (q & 1), jj = j + (q >> 1);
            if (ii < L.nx && jj < L.ny) vend[q] = L.at(ii, jj, kend);
        }
    }
#pragma unroll
    for (int u = 0; u < kMcGroup; ++u) {
        const int k = 32 * (w0 + u) + lane;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int ii = i + (q & 1), jj = j + (q >> 1);
            const bool in = ii < L.nx && jj < L.ny && k < L.nz;
            C[u].v[q] = v[u][q];
            C[u].up[q] = __ballot_sync(0xffffffffu, in && v[u][q] >= L.level);
        }
    }
    // the point after each chunk: lane 0 of the next chunk, or the loads at kend
    uint32_t nb_end = 0u;
    if (lane == 31 && kend < L.nz) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int ii = i + (q & 1), jj = j + (q >> 1);
            if (ii < L.nx && jj < L.ny) nb_end |= (uint32_t)(vend[q] >= L.level) << q;
        }
    }
    nb_end = __shfl_sync(0xffffffffu, nb_end, 31);
#pragma unroll
    for (int u = 0; u < kMcGroup; ++u) {
        if (u + 1 < kMcGroup) {
            uint32_t nb = 0u;
#pragma unroll
            for (int q = 0; q < 4; ++q) nb |= (C[u + 1].up[q] & 1u) << q;
            C[u].next = nb;
            C[u].v_next = __shfl_sync(0xffffffffu, v[u + 1][0], 0);
        } else {
            C[u].next = nb_end;
            C[u].v_next = vend[0];
        }
    }
}

// crossing masks of row (i, j) for the chunk at kb (bits of points k < nz only)
__device__ __forceinline__ void row_masks(const Lattice &L, int i, int j, int kb, const Chunk &C, uint32_t (&m)[3]) {
    const int left = L.nz - kb;   // points of this chunk in the lattice
    const uint32_t valid = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
    m[0] = i + 1 < L.nx ? (C.up[0] ^ C.up[1]) & valid : 0u;
    m[1] = j + 1 < L.ny ? (C.up[0] ^ C.up[2]) & valid : 0u;
    // z edge k -> k + 1 exists for k + 1 < nz
    const uint32_t zvalid = left - 1 >= 32 ? 0xffffffffu : (left - 1 > 0 ? ((1u << (left - 1)) - 1u) : 0u);
    m[2] = (C.up[0] ^ ((C.up[0] >> 1) | ((C.next & 1u) << 31))) & zvalid;
}

// the case of cube (i, j, kb + lane): corner c = (x, y, z) bits
__device__ __forceinline__ int cube_case(const Chunk &C, int lane) {
    int cs = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t nxt = lane < 31 ? (C.up[q] >> (lane + 1)) & 1u : (C.next >> q) & 1u;
        cs |= (int)((C.up[q] >> lane) & 1u) << q;
        cs |= (int)nxt << (q + 4);
    }
    return cs;
}

__device__ __forceinline__ int warp_incl_scan(int x, int lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    return x;
}

__global__ void __launch_bounds__(32 * kMcWarps) mc_count_kernel(Lattice L, uint32_t *__restrict__ masks,
                                                                 int32_t *__restrict__ vcount,
                                                                 int32_t *__restrict__ tcount) {
    const int lane = threadIdx.x & 31;
    const int nw = (L.nz + 31) / 32, ng = (nw + kMcGroup - 1) / kMcGroup;
    const int64_t n_items = (int64_t)L.nx * L.ny * ng;
    for (int64_t it = (int64_t)blockIdx.x * kMcWarps + (threadIdx.x >> 5); it < n_items;
         it += (int64_t)gridDim.x * kMcWarps) {
        const int64_t r = it / ng;
        const int w0 = (int)(it % ng) * kMcGroup;
        const int i = (int)(r / L.ny), j = (int)(r % L.ny);
        Chunk C[kMcGroup];
        load_group(L, i, j, w0, lane, C);
#pragma unroll
        for (int u = 0; u < kMcGroup; ++u) {
            const int w = w0 + u, kb = 32 * w;
            if (w >= nw) break;
            uint32_t m[3];
            row_masks(L, i, j, kb, C[u], m);
            if (lane < 3) masks[(r * 3 + lane) * nw + w] = lane == 0 ? m[0] : (lane == 1 ? m[1] : m[2]);
            // a chunk whose four rows (and the points after them) are all on
            // one side of the level has no triangles
            const uint32_t u0 = C[u].up[0];
            const bool flat = (u0 == 0u || u0 == 0xffffffffu) && C[u].up[1] == u0 && C[u].up[2] == u0 &&
                              C[u].up[3] == u0 && (kb + 32 >= L.nz || C[u].next == (u0 ? 0xFu : 0u));
            int nt = 0;
            if (!flat) {
                if (i + 1 < L.nx && j + 1 < L.ny && kb + lane + 1 < L.nz) nt = c_tri[cube_case(C[u], lane)][0];
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) nt += __shfl_xor_sync(0xffffffffu, nt, d);
            }
            if (lane == 0) {
                vcount[r * nw + w] = __popc(m[0]) + __popc(m[1]) + __popc(m[2]);
                tcount[r * nw + w] = nt;
            }
        }
    }
}

__global__ void __launch_bounds__(32 * kMcWarps) mc_emit_kernel(
    Lattice L, const uint32_t *__restrict__ masks, const int64_t *__restrict__ voff,
    const int64_t *__restrict__ toff, float ox, float oy, float oz, float sx, float sy, float sz,
    float *__restrict__ verts, int64_t *__restrict__ faces) {
    const int lane = threadIdx.x & 31;
    const int nw = (L.nz + 31) / 32, ng = (nw + kMcGroup - 1) / kMcGroup;
    const int64_t n_items = (int64_t)L.nx * L.ny * ng;
    for (int64_t it = (int64_t)blockIdx.x * kMcWarps + (threadIdx.x >> 5); it < n_items;
         it += (int64_t)gridDim.x * kMcWarps) {
        const int64_t r = it / ng;
        const int w0 = (int)(it % ng) * kMcGroup;
        const int i = (int)(r / L.ny), j = (int)(r % L.ny);
        const bool cubes = faces != nullptr && i + 1 < L.nx && j + 1 < L.ny;
        const bool own = verts != nullptr;
        // chunks with output (from the scanned counts: lanes 0..4 hold the
        // vertex offsets of chunks w0 .. w0 + 4, lanes 8..12 the face offsets);
        // most of a lattice has none, and those groups load nothing else
        uint32_t work = 0u;
        {
            const int lu = lane & 7;
            int64_t o = 0;
            if (lane < 16 && lu <= kMcGroup && w0 + lu <= nw) o = (lane < 8 ? voff : toff)[r * nw + w0 + lu];
#pragma unroll
            for (int u = 0; u < kMcGroup; ++u) {
                const int64_t v0 = __shfl_sync(0xffffffffu, o, u), v1 = __shfl_sync(0xffffffffu, o, u + 1);
                const int64_t t0 = __shfl_sync(0xffffffffu, o, 8 + u), t1 = __shfl_sync(0xffffffffu, o, 9 + u);
                if (w0 + u < nw && ((own && v1 > v0) || (cubes && t1 > t0))) work |= 1u << u;
            }
        }
        if (work == 0u) continue;
        // per chunk u: lanes 0..11 load the mask word (row q = lane / 3, axis
        // lane % 3); lanes 12..15 the x word of the next chunk of row lane -
        // 12; lanes 16..19 the vertex offset of the chunk of row lane - 16
        // (the neighbour rows exist whenever the row has cubes)
        uint32_t words[kMcGroup];
        int64_t offs[kMcGroup];
        {
            const int q = lane < 12 ? lane / 3 : (lane < 16 ? lane - 12 : (lane < 20 ? lane - 16 : 0));
            const int64_t rq = r + (q & 1) * (int64_t)L.ny + (q >> 1);
            const bool need = q == 0 ? (own || cubes) : cubes;
#pragma unroll
            for (int u = 0; u < kMcGroup; ++u) {
                const int w = w0 + u;
                words[u] = 0u;
                offs[u] = 0;
                if (w >= nw || !need) continue;
                if (lane < 12) words[u] = masks[(rq * 3 + lane % 3) * nw + w];
                else if (lane < 16 && w + 1 < nw) words[u] = masks[(rq * 3) * nw + w + 1];
                else if (lane >= 16 && lane < 20) offs[u] = voff[rq * nw + w];
            }
        }
        Chunk CG[kMcGroup];
        load_group(L, i, j, w0, lane, CG);
#pragma unroll
        for (int u = 0; u < kMcGroup; ++u) {
            const int w = w0 + u, kb = 32 * w;
            if (w >= nw) break;
            if (!((work >> u) & 1u)) continue;
            const Chunk &C = CG[u];
            const uint32_t word = words[u];
            const int64_t off = offs[u];
            uint32_t W[4][3], NX[4];
            int64_t vo[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
#pragma unroll
                for (int a = 0; a < 3; ++a) W[q][a] = __shfl_sync(0xffffffffu, word, 3 * q + a);
                NX[q] = __shfl_sync(0xffffffffu, word, 12 + q);
                vo[q] = __shfl_sync(0xffffffffu, off, 16 + q);
            }
            // vertices of this chunk of row (i, j): up to three per lane, in (k, axis) order
            if (own) {
                const uint32_t below = (1u << lane) - 1u;
                int64_t id = vo[0] + __popc(W[0][0] & below) + __popc(W[0][1] & below) + __popc(W[0][2] & below);
                const float vz = __shfl_down_sync(0xffffffffu, C.v[0], 1);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if ((W[0][a] >> lane) & 1u) {
                        const float v0 = C.v[0];
                        const float v1 = a == 0 ? C.v[1] : (a == 1 ? C.v[2] : (lane < 31 ? vz : C.v_next));
                        const float t = __fdiv_rn(__fsub_rn(L.level, v0), __fsub_rn(v1, v0));
                        float p[3] = {(float)i, (float)j, (float)(kb + lane)};
                        p[a] = __fadd_rn(p[a], t);
                        float *out = verts + id * 3;
                        out[0] = __fadd_rn(ox, __fmul_rn(p[0], sx));
                        out[1] = __fadd_rn(oy, __fmul_rn(p[1], sy));
                        out[2] = __fadd_rn(oz, __fmul_rn(p[2], sz));
                        ++id;
                    }
                }
            }
            // faces of this chunk's cubes, in cube order
            if (cubes) {
                // per (row q, z offset dz) with key = 2 q + dz: the vertex id of
                // the x edge at bit lane + dz, and that bit of the x and y masks
                // (the y and z edges at the same point follow it)
                int64_t base[8];
                uint32_t xb = 0u, yb = 0u;
                const uint32_t below0 = (1u << lane) - 1u;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint32_t all0 = __popc(W[q][0] & below0) + __popc(W[q][1] & below0) + __popc(W[q][2] & below0);
                    const uint32_t at0 = (W[q][0] >> lane) & 1u, at1 = (W[q][1] >> lane) & 1u,
                                   at2 = (W[q][2] >> lane) & 1u;
                    base[2 * q] = vo[q] + all0;
                    base[2 * q + 1] = vo[q] + all0 + at0 + at1 + at2;
                    xb |= at0 << (2 * q);
                    yb |= at1 << (2 * q);
                    const uint32_t nx0 = lane < 31 ? (W[q][0] >> (lane + 1)) & 1u : NX[q] & 1u;
                    const uint32_t ny0 = lane < 31 ? (W[q][1] >> (lane + 1)) & 1u : 0u;
                    xb |= nx0 << (2 * q + 1);
                    yb |= ny0 << (2 * q + 1);
                }
                const bool in = kb + lane + 1 < L.nz;
                const int8_t *row = c_tri[in ? cube_case(C, lane) : 0];
                const int nt = in ? row[0] : 0;
                const int incl = warp_incl_scan(nt, lane);
                int64_t f = toff[r * nw + w] + (incl - nt);
                for (int t = 0; t < nt; ++t, ++f) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const int e = row[1 + 3 * t + c];
                        const int a = e >> 2, m = e & 3;
                        // the lattice edge: axis a from (i + dx, j + dy, k + dz)
                        const int dx = a == 0 ? 0 : (m & 1);
                        const int dy = a == 0 ? (m & 1) : (a == 1 ? 0 : (m >> 1));
                        const int dz = a == 2 ? 0 : (m >> 1);
                        const int key = 2 * (dx | (dy << 1)) + dz;
                        int64_t id = base[0];
#pragma unroll
                        for (int u = 1; u < 8; ++u) id = key == u ? base[u] : id;
                        if (a >= 1) id += (xb >> key) & 1u;
                        if (a >= 2) id += (yb >> key) & 1u;
                        faces[f * 3 + c] = id;
                    }
                }
            }
        }
    }
}

// work items spread over at most the blocks resident at once
unsigned items_grid(int64_t n_items, const PersistentLaunch &c) {
    const int64_t b = (n_items + kMcWarps - 1) / kMcWarps;
    const int64_t cap = (int64_t)c.per_sm * c.sms;
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

struct McWorkspace {
    uint32_t *masks;
    int32_t *vcount, *tcount;
    int64_t *voff, *toff;
    void *scan;
};

struct McSizes {
    int64_t masks, counts, offs, scan;
};

McSizes mc_sizes(int32_t nx, int32_t ny, int32_t nz) {
    const int64_t rows = (int64_t)nx * ny, nw = (nz + 31) / 32, items = rows * nw;
    auto r = [](int64_t b) { return (b + 255) / 256 * 256; };
    return McSizes{r(rows * 3 * nw * 4), r(items * 4), r((items + 1) * 8), r(angelo_scan_workspace_size(items))};
}

McWorkspace carve(void *ws, int32_t nx, int32_t ny, int32_t nz) {
    const McSizes z = mc_sizes(nx, ny, nz);
    char *p = reinterpret_cast<char *>(ws);
    McWorkspace W;
    W.masks = reinterpret_cast<uint32_t *>(p);
    p += z.masks;
    W.vcount = reinterpret_cast<int32_t *>(p);
    p += z.counts;
    W.tcount = reinterpret_cast<int32_t *>(p);
    p += z.counts;
    W.voff = reinterpret_cast<int64_t *>(p);
    p += z.offs;
    W.toff = reinterpret_cast<int64_t *>(p);
    p += z.offs;
    W.scan = p;
    return W;
}

}  // namespace

extern "C" int64_t angelo_mc_workspace_size(int32_t nx, int32_t ny, int32_t nz) {
    if (nx < 2 || ny < 2 || nz < 2) return -1;
    const McSizes z = mc_sizes(nx, ny, nz);
    return z.masks + 2 * z.counts + 2 * z.offs + z.scan;
}

extern "C" int angelo_mc_count(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level, void *workspace,
                               int64_t *totals, void *stream) {
    ANGELO_REQUIRE(grid && workspace && totals, "mc_count: null pointer");
    ANGELO_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "mc_count: lattice %d x %d x %d", nx, ny, nz);
    if (int rc = ensure_table()) return rc;
    cudaStream_t s = as_stream(stream);
    const int64_t items = (int64_t)nx * ny * ((nz + 31) / 32);
    const int64_t groups = (int64_t)nx * ny * (((nz + 31) / 32 + kMcGroup - 1) / kMcGroup);
    McWorkspace W = carve(workspace, nx, ny, nz);
    Lattice L{grid, nx, ny, nz, level};
    static PersistentLaunch cfg;
    int rc = persistent_setup(mc_count_kernel, 0, 32 * kMcWarps, cfg, "mc_count");
    if (rc) return rc;
    mc_count_kernel<<<items_grid(groups, cfg), 32 * kMcWarps, 0, s>>>(L, W.masks, W.vcount, W.tcount);
    rc = check_launch("mc_count");
    if (rc) return rc;
    if ((rc = angelo_scan(W.vcount, items, W.voff, W.scan, stream))) return rc;
    if ((rc = angelo_scan(W.tcount, items, W.toff, W.scan, stream))) return rc;
    if (cudaMemcpyAsync(totals, W.voff + items, 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(totals + 1, W.toff + items, 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return check_launch("mc_count(totals)");
    return ANGELO_OK;
}

extern "C" int angelo_mc_extract(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level,
                                 const float *origin3, const float *spacing3, const void *workspace, float *vertices,
                                 int64_t *faces, void *stream) {
    ANGELO_REQUIRE(grid && workspace && origin3 && spacing3, "mc_extract: null pointer");
    ANGELO_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "mc_extract: lattice %d x %d x %d", nx, ny, nz);
    if (int rc = ensure_table()) return rc;
    if (!vertices && !faces) return ANGELO_OK;
    cudaStream_t s = as_stream(stream);
    const int64_t groups = (int64_t)nx * ny * (((nz + 31) / 32 + kMcGroup - 1) / kMcGroup);
    McWorkspace W = carve(const_cast<void *>(workspace), nx, ny, nz);
    Lattice L{grid, nx, ny, nz, level};
    static PersistentLaunch cfg;
    if (int rc = persistent_setup(mc_emit_kernel, 0, 32 * kMcWarps, cfg, "mc_extract")) return rc;
    mc_emit_kernel<<<items_grid(groups, cfg), 32 * kMcWarps, 0, s>>>(
        L, W.masks, W.voff, W.toff, origin3[0], origin3[1], origin3[2], spacing3[0], spacing3[1], spacing3[2],
        vertices, faces);
    return check_launch("mc_extract");
}
