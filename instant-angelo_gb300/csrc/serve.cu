// Native serving of a trained NeuS field: novel-view renders and SDF queries
// through fixed-shape buckets (the serving form of the eval path that the
// reference runs as NeuSModel.forward in 2048-ray chunks moved to the host,
// models/neus.py:285-293 with models/utils.py:14-51).
//
// A server holds the resident field (caller-owned device pointers: hash
// table, prepared MLP operands, occupancy bits) and one bucket's buffers.  A
// render bucket of B rays is: clip to the near/far planes or the scene box ->
// march count -> scan -> fill into the fixed sample capacity -> offsets
// clamped to it -> sample positions -> fused VolumeSDF (point + 6 FD taps,
// feature) -> fused radiance -> fused compositing (with the background).
// Nothing in it synchronises with the host, so it is captured once as a CUDA
// graph and replayed on the caller's stream for every bucket.  A bucket whose
// samples overflow the capacity is rendered again at its exact size (same
// kernels) after the call's buckets ran: the one host synchronisation of a
// render call.
#include <math.h>

#include <algorithm>
#include <new>

#include "common.cuh"

using namespace angelo;

struct angelo_server {
    angelo_serve_field f;
    int64_t B = 0, cap = 0, PB = 0;
    int use_graph = 0;
    // bucket inputs and march state
    float *ro = nullptr, *rd = nullptr, *tmin = nullptr, *tmax = nullptr;
    int32_t *counts = nullptr, *status = nullptr, *ri = nullptr;
    int64_t *offsets = nullptr;
    void *scan_ws = nullptr;
    float *t0 = nullptr, *t1 = nullptr, *pos = nullptr;
    // shading
    float *sdf = nullptr, *grad = nullptr, *feat = nullptr, *rgb = nullptr, *sdf_ws = nullptr;
    float *opacity = nullptr, *depth = nullptr, *comp = nullptr, *cnormal = nullptr, *full = nullptr,
          *accn = nullptr, *weights = nullptr, *trans = nullptr;
    float *aabb = nullptr;
    // SDF query workspace (points_per_bucket)
    float *q_ws = nullptr;
    // one status word per bucket of the current render call
    int32_t *bucket_status = nullptr;
    int64_t n_bucket_status = 0;
    int32_t *host_status = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    int device = -1;
};

namespace {

// nerfacc's t range without a scene box: [max(0, near), min(1e10, far)]
// (the planes of NeuSModel when set; a negative plane is "not set")
__global__ void planes_kernel(int64_t n, float near_plane, float far_plane, float *tmin, float *tmax) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tmin[i] = near_plane >= 0.f ? fmaxf(0.f, near_plane) : 0.f;
    tmax[i] = far_plane >= 0.f ? fminf(1e10f, far_plane) : 1e10f;
}

// sample positions o + d * (t0 + t1) / 2 in the order of torch's elementwise
// ops (add, multiply by 0.5, multiply by d, add o: each rounded)
__global__ void positions_kernel(const float *__restrict__ o, const float *__restrict__ d,
                                 const int32_t *__restrict__ ri, const float *__restrict__ t0,
                                 const float *__restrict__ t1, const int64_t *__restrict__ total,
                                 int64_t cap, float *__restrict__ pos) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = min(*total, cap);
    if (j >= n) return;
    const int64_t r = ri[j];
    const float mid = __fmul_rn(__fadd_rn(t0[j], t1[j]), 0.5f);
#pragma unroll
    for (int k = 0; k < 3; ++k) pos[j * 3 + k] = __fadd_rn(o[r * 3 + k], __fmul_rn(d[r * 3 + k], mid));
}

// rays [n, B) of a partial bucket: origin 0, direction +x (they march like
// any ray; their outputs are not copied out)
__global__ void pad_rays_kernel(int64_t n, int64_t B, float *o, float *d) {
    const int64_t i = n + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    o[i * 3 + 0] = o[i * 3 + 1] = o[i * 3 + 2] = 0.f;
    d[i * 3 + 0] = 1.f;
    d[i * 3 + 1] = d[i * 3 + 2] = 0.f;
}

bool planes_set(const angelo_serve_field &f) { return f.near_plane >= 0.f || f.far_plane >= 0.f; }

template <typename T>
int dalloc(T **p, int64_t n) {
    *p = nullptr;
    if (n <= 0) return ANGELO_OK;
    if (cudaMalloc(reinterpret_cast<void **>(p), (size_t)n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        set_error("serve: cudaMalloc of %lld bytes failed", (long long)(n * (int64_t)sizeof(T)));
        return ANGELO_E_CUDA;
    }
    return ANGELO_OK;
}

#define SERVE_TRY(x)                       \
    do {                                   \
        const int rc_ = (x);               \
        if (rc_ != ANGELO_OK) return rc_;  \
    } while (0)

// one render of n_rays rays in o/d (bucket buffers or exact-size buffers)
// with sample capacity cap; every pointer the caller's
struct RenderBufs {
    const float *o, *d;
    float *tmin, *tmax;
    int32_t *counts, *status, *ri;
    int64_t *offsets;
    void *scan_ws;
    float *t0, *t1, *pos, *sdf, *grad, *feat, *rgb, *sdf_ws;
    float *opacity, *depth, *comp, *cnormal, *full, *accn, *weights, *trans;
};

int march_and_shade(const angelo_server &S, const RenderBufs &b, int64_t n_rays, int64_t cap, bool clamp,
                    cudaStream_t st) {
    const angelo_serve_field &f = S.f;
    void *s = reinterpret_cast<void *>(st);
    if (planes_set(f)) {
        planes_kernel<<<blocks_for(n_rays, 256), 256, 0, st>>>(n_rays, f.near_plane, f.far_plane, b.tmin, b.tmax);
        SERVE_TRY(check_launch("serve: planes"));
    } else {
        SERVE_TRY(angelo_ray_aabb(b.o, b.d, n_rays, S.aabb, b.tmin, b.tmax, s));
    }
    SERVE_TRY(angelo_march_count(b.o, b.d, b.tmin, b.tmax, n_rays, &f.grid, f.render_step, 0.f, f.max_steps,
                                 b.counts, b.status, s));
    SERVE_TRY(angelo_scan(b.counts, n_rays, b.offsets, b.scan_ws, s));
    SERVE_TRY(angelo_march_fill(b.o, b.d, b.tmin, b.tmax, n_rays, &f.grid, f.render_step, 0.f, f.max_steps,
                                b.offsets, cap, b.ri, b.t0, b.t1, b.status, s));
    if (clamp) SERVE_TRY(angelo_offsets_clamp(b.offsets, n_rays, cap, s));
    positions_kernel<<<blocks_for(cap, 256), 256, 0, st>>>(b.o, b.d, b.ri, b.t0, b.t1, b.offsets + n_rays, cap,
                                                          b.pos);
    SERVE_TRY(check_launch("serve: positions"));
    // the fused stages run over the whole capacity: samples past the march's
    // total are padding (finite inputs: zeroed t, position 0) whose results
    // no ray's offsets reach
    const int od = f.sdf_layout.out_dim;
    SERVE_TRY(angelo_sdf_stencil_fwd(&f.lay, f.active_levels, f.table, f.table_dtype, &f.sdf_layout, f.sdf_net,
                                     b.pos, nullptr, cap, f.radius, f.eps, 1, 0, 1, b.sdf, b.grad, b.feat,
                                     od + 3, nullptr, b.sdf_ws, s));
    SERVE_TRY(angelo_radiance_fwd(f.feat_dim, f.rad_net, b.feat, od + 3, b.grad, b.ri, b.d, cap, f.rad_flags,
                                  b.rgb, s));
    SERVE_TRY(angelo_composite_fwd(b.offsets, n_rays, b.sdf, b.grad, b.t0, b.t1, b.d, b.rgb, f.variance,
                                   f.cos_anneal_ratio, f.background, 1e-4f, 2048.0f, b.opacity, b.depth,
                                   b.comp, b.cnormal, b.full, b.accn, b.weights, b.trans, nullptr, s));
    return ANGELO_OK;
}

RenderBufs bucket_bufs(const angelo_server &S) {
    return RenderBufs{S.ro,  S.rd,   S.tmin,    S.tmax,   S.counts,  S.status,  S.ri,   S.offsets,
                      S.scan_ws, S.t0, S.t1,    S.pos,    S.sdf,     S.grad,    S.feat, S.rgb,
                      S.sdf_ws, S.opacity, S.depth, S.comp, S.cnormal, S.full, S.accn, S.weights, S.trans};
}

int bucket_body(const angelo_server &S, cudaStream_t st) {
    if (cudaMemsetAsync(S.status, 0, sizeof(int32_t), st) != cudaSuccess) return check_launch("serve: status");
    return march_and_shade(S, bucket_bufs(S), S.B, S.cap, true, st);
}

void free_server(angelo_server *S) {
    if (!S) return;
    if (S->graph) cudaGraphExecDestroy(S->graph);
    if (S->cap_stream) cudaStreamDestroy(S->cap_stream);
    void *bufs[] = {S->ro,   S->rd,      S->tmin,  S->tmax,  S->counts, S->status,  S->ri,   S->offsets,
                    S->scan_ws, S->t0,   S->t1,    S->pos,   S->sdf,    S->grad,    S->feat, S->rgb,
                    S->sdf_ws, S->opacity, S->depth, S->comp, S->cnormal, S->full, S->accn, S->weights,
                    S->trans, S->aabb,   S->q_ws,  S->bucket_status};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (S->host_status) cudaFreeHost(S->host_status);
    delete S;
}

int alloc_bucket(angelo_server *S) {
    const int64_t B = S->B, C = S->cap;
    const int od = S->f.sdf_layout.out_dim;
    SERVE_TRY(dalloc(&S->ro, 3 * B));
    SERVE_TRY(dalloc(&S->rd, 3 * B));
    SERVE_TRY(dalloc(&S->tmin, B));
    SERVE_TRY(dalloc(&S->tmax, B));
    SERVE_TRY(dalloc(&S->counts, B));
    SERVE_TRY(dalloc(&S->status, 1));
    SERVE_TRY(dalloc(&S->offsets, B + 1));
    SERVE_TRY(dalloc(reinterpret_cast<char **>(&S->scan_ws), angelo_scan_workspace_size(B)));
    SERVE_TRY(dalloc(&S->ri, C));
    SERVE_TRY(dalloc(&S->t0, C));
    SERVE_TRY(dalloc(&S->t1, C));
    SERVE_TRY(dalloc(&S->pos, 3 * C));
    SERVE_TRY(dalloc(&S->sdf, C));
    SERVE_TRY(dalloc(&S->grad, 3 * C));
    SERVE_TRY(dalloc(&S->feat, (od + 3) * C));
    SERVE_TRY(dalloc(&S->rgb, 3 * C));
    SERVE_TRY(dalloc(&S->sdf_ws, angelo_sdf_workspace_floats(&S->f.lay, C, 1, 0, 0)));
    SERVE_TRY(dalloc(&S->opacity, B));
    SERVE_TRY(dalloc(&S->depth, B));
    SERVE_TRY(dalloc(&S->comp, 3 * B));
    SERVE_TRY(dalloc(&S->cnormal, 3 * B));
    SERVE_TRY(dalloc(&S->full, 3 * B));
    SERVE_TRY(dalloc(&S->accn, 3 * B));
    SERVE_TRY(dalloc(&S->weights, C));
    SERVE_TRY(dalloc(&S->trans, C));
    SERVE_TRY(dalloc(&S->aabb, 6));
    SERVE_TRY(dalloc(&S->q_ws, angelo_sdf_workspace_floats(&S->f.lay, S->PB, 0, 0, 0)));
    // padding samples past a bucket's total: finite t (the compositing and
    // positions never read them through a ray, but the fused stages run over
    // the whole capacity)
    if (cudaMemset(S->t0, 0, C * sizeof(float)) != cudaSuccess ||
        cudaMemset(S->t1, 0, C * sizeof(float)) != cudaSuccess ||
        cudaMemset(S->ri, 0, C * sizeof(int32_t)) != cudaSuccess ||
        cudaMemset(S->pos, 0, 3 * C * sizeof(float)) != cudaSuccess)
        return check_launch("serve: memset");
    const float r = S->f.radius;
    const float box[6] = {-r, -r, -r, r, r, r};
    if (cudaMemcpy(S->aabb, box, sizeof(box), cudaMemcpyHostToDevice) != cudaSuccess)
        return check_launch("serve: aabb");
    return ANGELO_OK;
}

int ensure_status(angelo_server *S, int64_t n_buckets) {
    if (n_buckets <= S->n_bucket_status) return ANGELO_OK;
    if (S->bucket_status) cudaFree(S->bucket_status);
    if (S->host_status) cudaFreeHost(S->host_status);
    S->bucket_status = nullptr;
    S->host_status = nullptr;
    S->n_bucket_status = 0;
    SERVE_TRY(dalloc(&S->bucket_status, n_buckets));
    if (cudaMallocHost(reinterpret_cast<void **>(&S->host_status), n_buckets * sizeof(int32_t)) != cudaSuccess) {
        cudaGetLastError();
        set_error("serve: cudaMallocHost failed");
        return ANGELO_E_CUDA;
    }
    S->n_bucket_status = n_buckets;
    return ANGELO_OK;
}

int d2d(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return ANGELO_OK;
    if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return check_launch("serve: copy");
    return ANGELO_OK;
}

// the exact-size render of rays [a, a + n) (the overflow path)
int render_exact(angelo_server *S, const float *rays_o, const float *rays_d, int64_t a, int64_t n, float *rgb,
                 float *opacity, float *depth, cudaStream_t st) {
    const angelo_serve_field &f = S->f;
    const int od = f.sdf_layout.out_dim;
    RenderBufs b{};
    b.o = rays_o + 3 * a;
    b.d = rays_d + 3 * a;
    int rc = ANGELO_OK;
    void *s = reinterpret_cast<void *>(st);
    int64_t total = 0;
    // pass 1 into temporaries: the exact sample count
    float *tmin = nullptr, *tmax = nullptr;
    int32_t *counts = nullptr, *status = nullptr;
    int64_t *offsets = nullptr;
    char *scan_ws = nullptr;
    auto cleanup = [&]() {
        void *ps[] = {tmin, tmax, counts, status, offsets, scan_ws};
        for (void *p : ps)
            if (p) cudaFree(p);
    };
    if ((rc = dalloc(&tmin, n)) || (rc = dalloc(&tmax, n)) || (rc = dalloc(&counts, n)) ||
        (rc = dalloc(&status, 1)) || (rc = dalloc(&offsets, n + 1)) ||
        (rc = dalloc(&scan_ws, angelo_scan_workspace_size(n)))) {
        cleanup();
        return rc;
    }
    if (planes_set(f)) {
        planes_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, f.near_plane, f.far_plane, tmin, tmax);
        rc = check_launch("serve: planes");
    } else {
        rc = angelo_ray_aabb(b.o, b.d, n, S->aabb, tmin, tmax, s);
    }
    if (!rc) rc = angelo_march_count(b.o, b.d, tmin, tmax, n, &f.grid, f.render_step, 0.f, f.max_steps, counts,
                                     status, s);
    if (!rc) rc = angelo_scan(counts, n, offsets, scan_ws, s);
    if (!rc && (cudaMemcpyAsync(&total, offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess))
        rc = check_launch("serve: exact total");
    cleanup();
    if (rc) return rc;
    const int64_t cap = std::max<int64_t>(total, 1);
    int32_t *ri = nullptr;
    float *t0 = nullptr, *t1 = nullptr, *pos = nullptr, *sdf = nullptr, *grad = nullptr, *feat = nullptr,
          *rgbs = nullptr, *sdf_ws = nullptr, *comp = nullptr, *cnormal = nullptr, *full = nullptr,
          *accn = nullptr, *weights = nullptr, *trans = nullptr, *op = nullptr, *dep = nullptr;
    auto cleanup2 = [&]() {
        void *ps[] = {tmin, tmax, counts, status, offsets, scan_ws, ri, t0, t1, pos, sdf, grad, feat, rgbs, sdf_ws,
                      comp, cnormal, full, accn, weights, trans, op, dep};
        for (void *p : ps)
            if (p) cudaFree(p);
    };
    tmin = tmax = nullptr;
    counts = status = nullptr;
    offsets = nullptr;
    scan_ws = nullptr;
    if ((rc = dalloc(&tmin, n)) || (rc = dalloc(&tmax, n)) || (rc = dalloc(&counts, n)) ||
        (rc = dalloc(&status, 1)) || (rc = dalloc(&offsets, n + 1)) ||
        (rc = dalloc(&scan_ws, angelo_scan_workspace_size(n))) || (rc = dalloc(&ri, cap)) ||
        (rc = dalloc(&t0, cap)) || (rc = dalloc(&t1, cap)) || (rc = dalloc(&pos, 3 * cap)) ||
        (rc = dalloc(&sdf, cap)) || (rc = dalloc(&grad, 3 * cap)) || (rc = dalloc(&feat, (od + 3) * cap)) ||
        (rc = dalloc(&rgbs, 3 * cap)) || (rc = dalloc(&sdf_ws, angelo_sdf_workspace_floats(&f.lay, cap, 1, 0, 0))) ||
        (rc = dalloc(&comp, 3 * n)) || (rc = dalloc(&cnormal, 3 * n)) || (rc = dalloc(&full, 3 * n)) ||
        (rc = dalloc(&accn, 3 * n)) || (rc = dalloc(&weights, cap)) || (rc = dalloc(&trans, cap)) ||
        (rc = dalloc(&op, n)) || (rc = dalloc(&dep, n))) {
        cleanup2();
        return rc;
    }
    if (cudaMemsetAsync(t0, 0, cap * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(t1, 0, cap * sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(ri, 0, cap * sizeof(int32_t), st) != cudaSuccess ||
        cudaMemsetAsync(pos, 0, 3 * cap * sizeof(float), st) != cudaSuccess)
        rc = check_launch("serve: exact memset");
    b.tmin = tmin;
    b.tmax = tmax;
    b.counts = counts;
    b.status = status;
    b.ri = ri;
    b.offsets = offsets;
    b.scan_ws = scan_ws;
    b.t0 = t0;
    b.t1 = t1;
    b.pos = pos;
    b.sdf = sdf;
    b.grad = grad;
    b.feat = feat;
    b.rgb = rgbs;
    b.sdf_ws = sdf_ws;
    b.opacity = op;
    b.depth = dep;
    b.comp = comp;
    b.cnormal = cnormal;
    b.full = full;
    b.accn = accn;
    b.weights = weights;
    b.trans = trans;
    if (!rc) rc = march_and_shade(*S, b, n, cap, false, st);
    if (!rc) rc = d2d(rgb + 3 * a, full, 3 * n * sizeof(float), st);
    if (!rc) rc = d2d(opacity + a, op, n * sizeof(float), st);
    if (!rc) rc = d2d(depth + a, dep, n * sizeof(float), st);
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = check_launch("serve: exact render");
    cleanup2();
    return rc;
}

}  // namespace

extern "C" int64_t angelo_serve_field_bytes(void) { return (int64_t)sizeof(angelo_serve_field); }

extern "C" int angelo_serve_create(const angelo_serve_field *field, int64_t rays_per_bucket,
                                   int32_t samples_per_ray, int64_t points_per_bucket, int32_t use_graph,
                                   angelo_server **out) {
    ANGELO_REQUIRE(field && out, "serve_create: null argument");
    *out = nullptr;
    ANGELO_REQUIRE(rays_per_bucket >= 1 && rays_per_bucket <= (1 << 24) && samples_per_ray >= 1 &&
                       points_per_bucket >= 1 && points_per_bucket <= (1ll << 26),
                   "serve_create: bucket shape");
    ANGELO_REQUIRE(rays_per_bucket * (int64_t)samples_per_ray <= (1ll << 28), "serve_create: sample capacity");
    ANGELO_REQUIRE(field->table && field->sdf_net && field->rad_net && field->variance && field->background,
                   "serve_create: null field pointer");
    ANGELO_REQUIRE(field->feat_dim == field->sdf_layout.out_dim + 3,
                   "serve_create: radiance feature width %d != sdf feature width %d", field->feat_dim,
                   field->sdf_layout.out_dim + 3);
    angelo_server *S = new (std::nothrow) angelo_server();
    ANGELO_REQUIRE(S, "serve_create: out of host memory");
    S->f = *field;
    S->B = rays_per_bucket;
    S->cap = rays_per_bucket * samples_per_ray;
    S->PB = points_per_bucket;
    S->use_graph = use_graph != 0;
    cudaGetDevice(&S->device);
    int rc = alloc_bucket(S);
    if (!rc && cudaStreamCreateWithFlags(&S->cap_stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = check_launch("serve_create: stream");
    // one run outside capture: kernel attributes and launch configurations
    // are set up before the capture
    if (!rc) rc = bucket_body(*S, S->cap_stream);
    if (!rc && cudaStreamSynchronize(S->cap_stream) != cudaSuccess) rc = check_launch("serve_create: warm-up");
    if (!rc && S->use_graph) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(S->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            rc = check_launch("serve_create: begin capture");
        } else {
            const int brc = bucket_body(*S, S->cap_stream);
            const cudaError_t e = cudaStreamEndCapture(S->cap_stream, &g);
            if (brc) rc = brc;
            else if (e != cudaSuccess) rc = check_launch("serve_create: end capture");
            else if (cudaGraphInstantiate(&S->graph, g, 0) != cudaSuccess) rc = check_launch("serve_create: instantiate");
            if (g) cudaGraphDestroy(g);
        }
    }
    if (rc) {
        free_server(S);
        return rc;
    }
    *out = S;
    return ANGELO_OK;
}

extern "C" int angelo_serve_render(angelo_server *S, const float *rays_o, const float *rays_d, int64_t n,
                                   float *rgb, float *opacity, float *depth, int64_t *overflows, void *stream) {
    ANGELO_REQUIRE(S, "serve_render: null server");
    ANGELO_REQUIRE(n >= 0, "serve_render: negative n");
    if (overflows) *overflows = 0;
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(rays_o && rays_d && rgb && opacity && depth, "serve_render: null pointer");
    cudaStream_t st = as_stream(stream);
    const int64_t nb = (n + S->B - 1) / S->B;
    SERVE_TRY(ensure_status(S, nb));
    for (int64_t k = 0; k < nb; ++k) {
        const int64_t a = k * S->B, m = std::min<int64_t>(S->B, n - a);
        SERVE_TRY(d2d(S->ro, rays_o + 3 * a, 3 * m * sizeof(float), st));
        SERVE_TRY(d2d(S->rd, rays_d + 3 * a, 3 * m * sizeof(float), st));
        if (m < S->B) {
            pad_rays_kernel<<<blocks_for(S->B - m, 256), 256, 0, st>>>(m, S->B, S->ro, S->rd);
            SERVE_TRY(check_launch("serve_render: pad"));
        }
        if (S->graph) {
            if (cudaGraphLaunch(S->graph, st) != cudaSuccess) return check_launch("serve_render: graph launch");
        } else {
            SERVE_TRY(bucket_body(*S, st));
        }
        SERVE_TRY(d2d(rgb + 3 * a, S->full, 3 * m * sizeof(float), st));
        SERVE_TRY(d2d(opacity + a, S->opacity, m * sizeof(float), st));
        SERVE_TRY(d2d(depth + a, S->depth, m * sizeof(float), st));
        SERVE_TRY(d2d(S->bucket_status + k, S->status, sizeof(int32_t), st));
    }
    if (cudaMemcpyAsync(S->host_status, S->bucket_status, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("serve_render: status");
    int64_t ovf = 0;
    for (int64_t k = 0; k < nb; ++k) {
        if (!(S->host_status[k] & 2)) continue;
        ++ovf;
        const int64_t a = k * S->B, m = std::min<int64_t>(S->B, n - a);
        SERVE_TRY(render_exact(S, rays_o, rays_d, a, m, rgb, opacity, depth, st));
    }
    if (overflows) *overflows = ovf;
    return ANGELO_OK;
}

extern "C" int angelo_serve_sdf(angelo_server *S, const float *points, int64_t n, float *sdf, void *stream) {
    ANGELO_REQUIRE(S, "serve_sdf: null server");
    ANGELO_REQUIRE(n >= 0, "serve_sdf: negative n");
    if (n == 0) return ANGELO_OK;
    ANGELO_REQUIRE(points && sdf, "serve_sdf: null pointer");
    const angelo_serve_field &f = S->f;
    for (int64_t a = 0; a < n; a += S->PB) {
        const int64_t m = std::min<int64_t>(S->PB, n - a);
        SERVE_TRY(angelo_sdf_stencil_fwd(&f.lay, f.active_levels, f.table, f.table_dtype, &f.sdf_layout, f.sdf_net,
                                         points + 3 * a, nullptr, m, f.radius, f.eps, 0, 0, 0, sdf + a, nullptr,
                                         nullptr, 0, nullptr, S->q_ws, stream));
    }
    return ANGELO_OK;
}

extern "C" int angelo_serve_destroy(angelo_server *S) {
    if (!S) return ANGELO_OK;
    if (S->device >= 0) cudaSetDevice(S->device);
    cudaDeviceSynchronize();
    free_server(S);
    return ANGELO_OK;
}
