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
// Passes: edge counts -> scan -> vertices; cube triangle counts -> scan ->
// faces (vertex indices through the edge scan).
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

struct Lattice {
    const float *v;
    int nx, ny, nz;
    float level;
    __device__ __forceinline__ float at(int64_t i, int64_t j, int64_t k) const { return v[(i * ny + j) * nz + k]; }
};

// edge e of lattice point p: axis e % 3 from p; counts 1 when it crosses the level
__global__ void mc_edge_count_kernel(Lattice L, int32_t *__restrict__ counts) {
    const int64_t n = (int64_t)L.nx * L.ny * L.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = e / 3;
        const int a = (int)(e % 3);
        const int64_t i = p / ((int64_t)L.ny * L.nz), j = (p / L.nz) % L.ny, k = p % L.nz;
        int c = 0;
        if ((a == 0 && i + 1 < L.nx) || (a == 1 && j + 1 < L.ny) || (a == 2 && k + 1 < L.nz)) {
            const float v0 = L.at(i, j, k);
            const float v1 = L.at(i + (a == 0), j + (a == 1), k + (a == 2));
            c = (v0 >= L.level) != (v1 >= L.level);
        }
        counts[e] = c;
    }
}

__global__ void mc_vertex_kernel(Lattice L, const int32_t *__restrict__ counts, const int64_t *__restrict__ offs,
                                 float ox, float oy, float oz, float sx, float sy, float sz,
                                 float *__restrict__ verts) {
    const int64_t n = (int64_t)L.nx * L.ny * L.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += (int64_t)gridDim.x * blockDim.x) {
        if (!counts[e]) continue;
        const int64_t p = e / 3;
        const int a = (int)(e % 3);
        const int64_t i = p / ((int64_t)L.ny * L.nz), j = (p / L.nz) % L.ny, k = p % L.nz;
        const float v0 = L.at(i, j, k), v1 = L.at(i + (a == 0), j + (a == 1), k + (a == 2));
        const float t = __fdiv_rn(__fsub_rn(L.level, v0), __fsub_rn(v1, v0));
        float q[3] = {(float)i, (float)j, (float)k};
        q[a] = __fadd_rn(q[a], t);
        float *out = verts + offs[e] * 3;
        out[0] = __fadd_rn(ox, __fmul_rn(q[0], sx));
        out[1] = __fadd_rn(oy, __fmul_rn(q[1], sy));
        out[2] = __fadd_rn(oz, __fmul_rn(q[2], sz));
    }
}

__device__ __forceinline__ int cube_case(const Lattice &L, int64_t i, int64_t j, int64_t k) {
    int cs = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) cs |= (L.at(i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1)) >= L.level) << c;
    return cs;
}

__global__ void mc_cube_count_kernel(Lattice L, int32_t *__restrict__ counts) {
    const int64_t cx = L.nx - 1, cy = L.ny - 1, cz = L.nz - 1, n = cx * cy * cz;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = c / (cy * cz), j = (c / cz) % cy, k = c % cz;
        counts[c] = c_tri[cube_case(L, i, j, k)][0];
    }
}

// global id of local edge e of cube (i, j, k): the lattice edge of axis e / 4
// from corner edge_c[e][0]
__device__ __forceinline__ int64_t global_edge(const Lattice &L, int64_t i, int64_t j, int64_t k, int e) {
    const int a = e >> 2, m = e & 3;
    int64_t p[3] = {i, j, k};
    const int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
    p[o0] += m & 1;
    p[o1] += (m >> 1) & 1;
    return ((p[0] * L.ny + p[1]) * L.nz + p[2]) * 3 + a;
}

__global__ void mc_face_kernel(Lattice L, const int64_t *__restrict__ eoffs, const int64_t *__restrict__ coffs,
                               int64_t *__restrict__ faces) {
    const int64_t cx = L.nx - 1, cy = L.ny - 1, cz = L.nz - 1, n = cx * cy * cz;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f0 = coffs[c];
        if (coffs[c + 1] == f0) continue;
        const int64_t i = c / (cy * cz), j = (c / cz) % cy, k = c % cz;
        const int8_t *row = c_tri[cube_case(L, i, j, k)];
        for (int t = 0; t < row[0]; ++t)
            for (int q = 0; q < 3; ++q) faces[(f0 + t) * 3 + q] = eoffs[global_edge(L, i, j, k, row[1 + 3 * t + q])];
    }
}

unsigned grid_for(int64_t n) {
    const int64_t b = (n + 255) / 256;
    return (unsigned)(b < 65535 * 8 ? (b > 0 ? b : 1) : 65535 * 8);
}

struct McWorkspace {
    int32_t *ecounts;
    int64_t *eoffs;
    int32_t *ccounts;
    int64_t *coffs;
    void *scan;
};

int64_t scan_bytes(int64_t n);

McWorkspace carve(void *ws, int64_t n_points, int64_t n_cubes) {
    char *p = reinterpret_cast<char *>(ws);
    auto take = [&](int64_t bytes) {
        char *r = p;
        p += (bytes + 255) / 256 * 256;
        return r;
    };
    McWorkspace W;
    W.ecounts = reinterpret_cast<int32_t *>(take(3 * n_points * 4));
    W.eoffs = reinterpret_cast<int64_t *>(take((3 * n_points + 1) * 8));
    W.ccounts = reinterpret_cast<int32_t *>(take(n_cubes * 4));
    W.coffs = reinterpret_cast<int64_t *>(take((n_cubes + 1) * 8));
    W.scan = take(scan_bytes(3 * n_points > n_cubes ? 3 * n_points : n_cubes));
    return W;
}

int64_t scan_bytes(int64_t n) { return angelo_scan_workspace_size(n); }

}  // namespace

extern "C" int64_t angelo_mc_workspace_size(int32_t nx, int32_t ny, int32_t nz) {
    if (nx < 2 || ny < 2 || nz < 2) return -1;
    const int64_t n = (int64_t)nx * ny * nz, c = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
    auto r = [](int64_t b) { return (b + 255) / 256 * 256; };
    return r(3 * n * 4) + r((3 * n + 1) * 8) + r(c * 4) + r((c + 1) * 8) + r(scan_bytes(3 * n > c ? 3 * n : c));
}

extern "C" int angelo_mc_count(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level, void *workspace,
                               int64_t *totals, void *stream) {
    ANGELO_REQUIRE(grid && workspace && totals, "mc_count: null pointer");
    ANGELO_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "mc_count: lattice %d x %d x %d", nx, ny, nz);
    if (int rc = ensure_table()) return rc;
    cudaStream_t s = as_stream(stream);
    const int64_t n = (int64_t)nx * ny * nz, c = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
    McWorkspace W = carve(workspace, n, c);
    Lattice L{grid, nx, ny, nz, level};
    mc_edge_count_kernel<<<grid_for(3 * n), 256, 0, s>>>(L, W.ecounts);
    mc_cube_count_kernel<<<grid_for(c), 256, 0, s>>>(L, W.ccounts);
    int rc = check_launch("mc_count");
    if (rc) return rc;
    if ((rc = angelo_scan(W.ecounts, 3 * n, W.eoffs, W.scan, stream))) return rc;
    if ((rc = angelo_scan(W.ccounts, c, W.coffs, W.scan, stream))) return rc;
    if (cudaMemcpyAsync(totals, W.eoffs + 3 * n, 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(totals + 1, W.coffs + c, 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return check_launch("mc_count(totals)");
    return ANGELO_OK;
}

extern "C" int angelo_mc_extract(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level,
                                 const float *origin3, const float *spacing3, const void *workspace, float *vertices,
                                 int64_t *faces, void *stream) {
    ANGELO_REQUIRE(grid && workspace && origin3 && spacing3, "mc_extract: null pointer");
    ANGELO_REQUIRE(nx >= 2 && ny >= 2 && nz >= 2, "mc_extract: lattice %d x %d x %d", nx, ny, nz);
    if (int rc = ensure_table()) return rc;
    cudaStream_t s = as_stream(stream);
    const int64_t n = (int64_t)nx * ny * nz, c = (int64_t)(nx - 1) * (ny - 1) * (nz - 1);
    McWorkspace W = carve(const_cast<void *>(workspace), n, c);
    Lattice L{grid, nx, ny, nz, level};
    if (vertices)
        mc_vertex_kernel<<<grid_for(3 * n), 256, 0, s>>>(L, W.ecounts, W.eoffs, origin3[0], origin3[1], origin3[2],
                                                        spacing3[0], spacing3[1], spacing3[2], vertices);
    if (faces) mc_face_kernel<<<grid_for(c), 256, 0, s>>>(L, W.eoffs, W.coffs, faces);
    return check_launch("mc_extract");
}
