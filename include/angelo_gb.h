/*
 * angelo_gb.h -- C ABI of libangelo_gb.so, the sm_103a (GB300) kernels of the
 * NeuS / Neuralangelo hot path of Instant-angelo.
 *
 * Conventions
 *   - Every entry point is extern "C", takes plain device pointers, element
 *     counts and a cudaStream_t passed as void*, and returns an int status:
 *     ANGELO_OK (0) or one of ANGELO_E_*; angelo_last_error_string() returns a
 *     thread-local description of the last failure.  No C++ exception crosses
 *     the ABI.
 *   - Calls are stream-ordered and asynchronous; the library keeps no mutable
 *     global state and never allocates device memory: outputs and workspace
 *     belong to the caller (workspace sizes are queried per op).
 *   - Tensors are row-major.  Points/directions are float32 (n, 3).  A hash
 *     table is the tcnn flat parameter vector: entries of F=2 features, level
 *     l starting at entry offsets[l].
 *
 * Each declaration names the reference call it replaces (path:line in the
 * Instant-angelo tree).
 */
#ifndef ANGELO_GB_H
#define ANGELO_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ANGELO_OK 0
#define ANGELO_E_INVALID 1     /* bad argument: null pointer, size, alignment */
#define ANGELO_E_CUDA 2        /* CUDA launch or runtime error */
#define ANGELO_E_UNSUPPORTED 3 /* configuration outside what the kernels handle */
#define ANGELO_E_CAPACITY 4    /* an output would exceed its stated capacity */

#define ANGELO_MAX_LEVELS 32

#define ANGELO_DTYPE_F32 0
#define ANGELO_DTYPE_F16 1

/* Hash-grid description: the keys of the reference's xyz_encoding_config
 * (configs/neuralangelo-colmap_sparse.yaml:48-58). */
typedef struct {
    int32_t n_levels;          /* <= ANGELO_MAX_LEVELS */
    int32_t n_features;        /* must be 2 */
    int32_t log2_hashmap_size; /* <= 30 */
    int32_t base_resolution;
    float per_level_scale;
} angelo_hashgrid_desc;

/* Per-level layout derived from a description (tcnn's offset table). */
typedef struct {
    int32_t n_levels;
    int32_t n_features;
    uint32_t offsets[ANGELO_MAX_LEVELS + 1]; /* entry offset of every level, last = total */
    uint32_t resolutions[ANGELO_MAX_LEVELS];
    float scales[ANGELO_MAX_LEVELS];
} angelo_hashgrid_layout_t;

const char *angelo_last_error_string(void);
int angelo_version(void);

/* --------------------------------------------------------------- hash grid */

/* Layout of tcnn.Encoding(otype=HashGrid) (models/network_utils.py:47):
 * scale_l = exp2f(l*log2f(b))*base - 1, res_l = ceil(scale_l)+1,
 * entries_l = min(align8(res_l^3), 2^log2T).  Host only. */
int angelo_hashgrid_layout(const angelo_hashgrid_desc *desc, angelo_hashgrid_layout_t *out);

/* Encode forward, replaces ProgressiveBandHashGrid.forward
 * (models/network_utils.py:56-59) and CompositeEncoding.forward (:78-79).
 * x: (n,3) contracted points.  Writes, per point i, at out + i*out_stride +
 * out_col: [x*2-1 (3 values, only if include_xyz)] then L*2 features; levels
 * >= active_levels are written as 0 (band mask).  table_dtype: F32 or F16. */
int angelo_hashgrid_fwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                        const float *x, int64_t n, const void *table, int32_t table_dtype,
                        int32_t include_xyz, float *out, int64_t out_stride, int64_t out_col,
                        void *stream);

/* Encode backward (tcnn HashGrid backward behind the same call).
 * dout holds dL/d(encoding) with the same stride/column convention.
 * dtable (float32, may be NULL) is ACCUMULATED (atomic, order not fixed).
 * dx (n,3, may be NULL) is WRITTEN with dL/dx, including the xyz columns when
 * include_xyz; computing it reads table. */
int angelo_hashgrid_bwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                        const float *x, int64_t n, const void *table, int32_t table_dtype,
                        int32_t include_xyz, const float *dout, int64_t dout_stride,
                        int64_t dout_col, float *dtable, float *dx, void *stream);

/* Corner indices / weights of every (point, level): idx (n, L, 8) uint32
 * entry index inside the level, w (n, L, 8) float32.  Test hook for the
 * bit-exact index check. */
int angelo_hashgrid_index(const angelo_hashgrid_layout_t *lay, const float *x, int64_t n,
                          uint32_t *idx, float *w, void *stream);

/* ------------------------------------------------------ spherical harmonics */

/* Degree-4 real SH (16 values), replaces tcnn SphericalHarmonics reached
 * through get_encoding at models/texture.py:17,24-25.  With from_unit != 0 the
 * input is a unit direction d and the reference's (d+1)/2 mapping is applied
 * in the kernel; otherwise the input is already in [0,1]. */
int angelo_sh4_fwd(const float *dirs, int64_t n, int32_t from_unit, float *out,
                   int64_t out_stride, int64_t out_col, void *stream);
/* dL/ddirs (written) from dL/dout. */
int angelo_sh4_bwd(const float *dirs, int64_t n, int32_t from_unit, const float *dout,
                   int64_t dout_stride, int64_t dout_col, float *ddirs, void *stream);

/* ------------------------------------------------------------ ray marching */

/* nerfacc.intersection.ray_aabb_intersect (models/neus.py:12,153). */
int angelo_ray_aabb(const float *rays_o, const float *rays_d, int64_t n, const float *aabb6,
                    float *t_min, float *t_max, void *stream);

/* Occupancy grid as seen by the marcher: res^3 cells over roi, one bit per
 * cell, cell index = ix*res_y*res_z + iy*res_z + iz, bit (c & 31) of word
 * c >> 5.  A NULL bits pointer means "every cell occupied".  contraction
 * (nerfacc 0.3.3 ContractionType): ANGELO_CONTRACT_AABB, cells over roi and
 * nothing outside it, empty cells skipped to the next cell boundary; or
 * ANGELO_CONTRACT_UNBOUNDED_SPHERE (the learned background's grid,
 * models/neus.py:69-74), roi mapped to [-1,1]^3, points beyond the unit
 * sphere contracted to radius 2 - 1/|x|, the radius-2 ball to [0,1]^3, no
 * skipping. */
#define ANGELO_CONTRACT_AABB 0
#define ANGELO_CONTRACT_UNBOUNDED_SPHERE 1
typedef struct {
    float roi[6];
    int32_t res[3];
    const uint32_t *bits;
    int32_t contraction;
} angelo_grid_t;

/* nerfacc.ray_marching (models/neus.py:210-220), pass 1: samples per ray.
 * status (device int32, may be NULL) gets bit 0 set when a ray reaches
 * max_steps loop iterations. */
int angelo_march_count(const float *rays_o, const float *rays_d, const float *t_min,
                       const float *t_max, int64_t n_rays, const angelo_grid_t *grid,
                       float step, float cone_angle, int64_t max_steps, int32_t *counts,
                       int32_t *status, void *stream);

/* Exclusive scan of int32 counts into int64 offsets (n+1 values, last =
 * total).  Workspace: angelo_scan_workspace_size(n) bytes. */
int64_t angelo_scan_workspace_size(int64_t n);
int angelo_scan(const int32_t *counts, int64_t n, int64_t *offsets, void *workspace,
                void *stream);

/* Allocation-free exclusive scan: same result as angelo_scan, for callers
 * that cannot allocate device memory (a host that gives the library only
 * fixed, pre-sized buffers from its own pool, or code that may not call
 * cudaMalloc where it runs).  This entry point has no counterpart in the
 * reference.  Its workspace is a fixed 128 KiB array inside the library that
 * every GPU loading the library keeps until the process exits; n may be at
 * most ANGELO_SCAN_NOALLOC_MAX_N (larger n returns ANGELO_E_INVALID).  All
 * calls share that array: calls whose kernels overlap on the GPU race, so
 * order them on one stream.  Each call made outside stream capture looks up
 * the array's address with the calling device current (so a re-created
 * context is followed); a call under capture reuses the last address looked
 * up on that device, so make the first call on a device before any stream
 * capture (a first call under capture returns ANGELO_E_INVALID). */
#define ANGELO_SCAN_NOALLOC_MAX_N (1LL << 24)
int angelo_scan_noalloc(const int32_t *counts, int64_t n, int64_t *offsets, void *stream);

/* Pass 2: writes ray_indices (int32), t_starts, t_ends at offsets[i] + j.
 * Samples at or past capacity are dropped and status bit 1 is set. */
int angelo_march_fill(const float *rays_o, const float *rays_d, const float *t_min,
                      const float *t_max, int64_t n_rays, const angelo_grid_t *grid, float step,
                      float cone_angle, int64_t max_steps, const int64_t *offsets,
                      int64_t capacity, int32_t *ray_indices, float *t_starts, float *t_ends,
                      int32_t *status, void *stream);

/* offsets[0..n_rays] = min(offsets, capacity), in place.  After a
 * march_fill into a fixed capacity (which drops the samples at or past it),
 * this keeps every consumer that walks [offsets[r], offsets[r+1]) -- the
 * weights, accumulation and fused compositing -- inside the capacity; the
 * overflow itself stays flagged in the fill's status (bit 1).  No
 * counterpart in the reference (nerfacc sizes its outputs exactly). */
int angelo_offsets_clamp(int64_t *offsets, int64_t n_rays, int64_t capacity, void *stream);

/* Single-march variant of passes 1 and 2 (no counterpart in the reference;
 * same samples): march_record marches every ray once, writing its sample
 * count to counts and its first per_ray samples as (t_start, t_end) pairs to
 * scratch[2 * (ray * per_ray + j)]; a ray with more than per_ray samples sets
 * status bit 2 (use march_fill then).  After the scan, march_compact copies
 * the recorded samples to the packed outputs (capacity as in march_fill).
 * per_ray >= ceil(ray length / step) + 2 bounds every ray (each sample
 * advances t by at least step). */
int angelo_march_record(const float *rays_o, const float *rays_d, const float *t_min,
                        const float *t_max, int64_t n_rays, const angelo_grid_t *grid,
                        float step, float cone_angle, int64_t max_steps, int32_t per_ray,
                        float *scratch, int32_t *counts, int32_t *status, void *stream);
int angelo_march_compact(const float *scratch, int32_t per_ray, const int32_t *counts,
                         const int64_t *offsets, int64_t n_rays, int64_t capacity,
                         int32_t *ray_indices, float *t_starts, float *t_ends, int32_t *status,
                         void *stream);

/* ------------------------------------------------------- marching cubes */

/* Isosurface of an nx x ny x nz float32 lattice (x-major: value (i,j,k) at
 * (i*ny + j)*nz + k) at `level`, replacing PyMCubes in MarchingCubeHelper
 * (models/geometry.py:79-113; isosurface() triangulates the SDF at 0.001).
 * One vertex per lattice edge whose ends straddle the level (value >= level
 * on one end), linearly interpolated; triangles per cube from a 256-case
 * table built by a face-walk rule that cuts off the corners at or above the
 * level (the mesh is closed where the surface stays inside the lattice;
 * triangles face the higher values).  No counterpart table in the reference
 * (it calls PyMCubes): the vertex set is the same, the triangulation of
 * ambiguous faces may differ.
 * angelo_mc_count fills the workspace (angelo_mc_workspace_size bytes) and
 * writes the vertex and face totals to totals (device int64[2]);
 * angelo_mc_extract then writes vertices (totals[0] x 3 floats, origin +
 * index * spacing) and faces (totals[1] x 3 int64 vertex indices); either
 * output may be NULL. */
int64_t angelo_mc_workspace_size(int32_t nx, int32_t ny, int32_t nz);
int angelo_mc_count(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level,
                    void *workspace, int64_t *totals, void *stream);
int angelo_mc_extract(const float *grid, int32_t nx, int32_t ny, int32_t nz, float level,
                      const float *origin3, const float *spacing3, const void *workspace,
                      float *vertices, int64_t *faces, void *stream);

/* ------------------------------------------------------- occupancy update */

/* OccupancyGrid._update's EMA + threshold (models/neus.py:108-109 through
 * nerfacc 0.3.3): occs[c] = max(occs[c]*decay, max over the k with
 * cells[k]==c of occ[k]) for every sampled cell, then bits = occs >
 * min(mean(occs), thre).  Workspace: angelo_occ_workspace_size(n_cells). */
int64_t angelo_occ_workspace_size(int64_t n_cells);
int angelo_occ_update(float *occs, int64_t n_cells, const int64_t *cells, const float *occ,
                      int64_t k, float decay, float thre, uint32_t *bits, void *workspace,
                      void *stream);

/* -------------------------------------------------------------- compositing */

/* nerfacc.render_weight_from_alpha (models/neus.py:234): per ray in sample
 * order T_0 = 1, w_j = a_j*T_j, T_{j+1} = T_j*(1-a_j); w_j = 0 once T_j <
 * early_stop_eps.  trans (may be NULL) receives T_j. */
int angelo_weights_fwd(const float *alpha, const int64_t *offsets, int64_t n_rays,
                       float early_stop_eps, float *weights, float *trans, void *stream);
/* dL/dalpha (written) from dL/dweights and the forward's transmittance by the
 * reverse scan R_{j-1} = g_j a_j + (1-a_j) R_j, dalpha_j = T_j (g_j - R_j). */
int angelo_weights_bwd(const float *alpha, const float *trans, const int64_t *offsets,
                       int64_t n_rays, float early_stop_eps, const float *dweights,
                       float *dalpha, void *stream);

/* nerfacc.render_weight_from_density (the learned background,
 * models/neus.py:171): per ray in sample order, tau_j = sigma_j (t_end_j -
 * t_start_j), w_j = (1 - exp(-tau_j)) exp(-(tau_0 + .. + tau_{j-1})). */
int angelo_density_weights_fwd(const float *t_starts, const float *t_ends, const float *sigmas,
                               const int64_t *offsets, int64_t n_rays, float *weights, void *stream);
/* dsigmas (written) from dweights, with the forward's weights. */
int angelo_density_weights_bwd(const float *t_starts, const float *t_ends, const float *sigmas,
                               const float *weights, const int64_t *offsets, int64_t n_rays,
                               const float *dweights, float *dsigmas, void *stream);

/* nerfacc.accumulate_along_rays (models/neus.py:235-240): out[r, c] =
 * sum_j w_j * v[j, c] over the samples of ray r (v == NULL: v = 1, C = 1). */
int angelo_accumulate_fwd(const float *weights, const float *values, int32_t channels,
                          const int64_t *offsets, int64_t n_rays, float *out, void *stream);
/* dweights (written) and dvalues (written, may be NULL). */
int angelo_accumulate_bwd(const float *weights, const float *values, int32_t channels,
                          const int64_t *offsets, int64_t n_rays, const float *dout,
                          float *dweights, float *dvalues, void *stream);

/* ------------------------------------------------------------ fused VolumeSDF */

#define ANGELO_OPERAND_BF16 0
#define ANGELO_OPERAND_FP16 1

/* Prepared geometry-MLP operands: fp32 biases and output row 0, and the
 * three layers as bf16 (or fp16) hi/lo tensor-core operands.  Layout by
 * query. */
typedef struct {
    int32_t k_tiles1, n_hidden, n_tiles3, k_tiles3b, out_dim;
    int64_t off_b1, off_b2, off_b3, off_w3row0;
    /* tensor-core (tcgen05) operands: W1 (64 x 16*k_tiles1), W2 (64 x 64),
     * W3 (16*k_tiles3b x 64) in the K-major core-matrix layout, bf16 hi then lo */
    int64_t off_tcw1, off_tcw2, off_tcw3;
    int64_t bytes;
    /* tensor-core products per layer in the forward kernels: 3 (bf16x3, the
     * default the query sets: hi*hi + lo*hi + hi*lo, ~16 mantissa bits per
     * operand) or 1 (the hi parts alone, a single pass); the backward
     * recompute is always bf16x3 */
    int32_t mma_passes;
    /* number format of the prepared weights and of the forward kernels'
     * staged activations: ANGELO_OPERAND_BF16 (the default the query sets) or
     * ANGELO_OPERAND_FP16 (11 significant bits: with one pass, the precision
     * form).  Set it before angelo_sdf_prep; the backward accepts only a
     * bf16-prepared buffer. */
    int32_t operand_format;
} angelo_sdf_net_layout;

int angelo_sdf_net_layout_query(int32_t n_levels, int32_t n_hidden, int32_t out_dim,
                                angelo_sdf_net_layout *out);

/* Convert the effective fp32 weights of the reference's VanillaMLP
 * (models/network_utils.py:96-140, after weight normalisation; W row-major
 * (out, in), reference input order [x*2-1, hash]) into the prepared buffer.
 * W2/b2 are ignored with one hidden layer. */
int angelo_sdf_prep(const angelo_sdf_net_layout *lay, int32_t n_levels, int32_t in_dim,
                    const float *W1, const float *b1, const float *W2, const float *b2,
                    const float *W3, const float *b3, void *net, void *stream);

/* Number of floats of the flat weight gradient written by the backward:
 * [dW1 (64 x 16*k_tiles1, kernel column order: hash, xyz, pad), dW2 (64 x 64),
 *  dW3 (16*k_tiles3b x 64), db1 (64), db2 (64), db3 (16*k_tiles3b)]. */
int64_t angelo_sdf_grad_size(const angelo_sdf_net_layout *lay);

/* Floats of device workspace of the fused VolumeSDF for n samples: the
 * forward's (backward = 0: the hash encodings of every evaluation, level-major
 * float2, 16 floats of stencil state per sample and, with the curvature, the
 * derivative of each curvature tap's encoding along the three axes, 6 x
 * levels x 3 float2 per sample) or the backward's (backward = 1:
 * dL/d(encodings), same layout as the encodings, and 8 floats per sample).
 * -1 on invalid arguments.  Both must be 8-byte aligned. */
int64_t angelo_sdf_workspace_floats(const angelo_hashgrid_layout_t *lay, int64_t n,
                                    int32_t with_grad, int32_t with_laplace, int32_t backward);

/* Fused VolumeSDF.forward with grad_type='finite_difference'
 * (models/geometry.py:195-287): per sample the point, the 6-tap FD stencil
 * and the 6-tap curvature stencil (13 hash-grid + MLP evaluations), with the
 * reference's quirks (clamped stencil divided by 2 eps; curvature shift in
 * contracted coordinates then clamped as world coordinates).  pos: (n,3)
 * world points; rand_dirs: (n,3), the randn of models/geometry.py:238.
 * Outputs sdf (n), grad (n,3), feature (n, feat_stride >= out_dim+3:
 * [MLP output, x*2-1]), laplace (n).  workspace: the forward workspace
 * (angelo_sdf_workspace_floats(.., 0) floats); a training forward keeps it,
 * unmodified, for the backward.  Instantiated network shapes: 8 levels /
 * 1 hidden layer / 9..16 outputs and 16 levels / 2 hidden layers / 65..72
 * outputs (angelo_sdf_net_layout_query refuses others). */
int angelo_sdf_stencil_fwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                           const void *table, int32_t table_dtype, const angelo_sdf_net_layout *nl,
                           const void *net, const float *pos, const float *rand_dirs, int64_t n,
                           float radius, float eps, int32_t with_grad, int32_t with_laplace,
                           int32_t with_feature, float *sdf, float *grad, float *feature,
                           int64_t feat_stride, float *laplace, float *workspace, void *stream);

/* Backward of the fused VolumeSDF: from dL/dsdf, dL/dgrad, dL/dfeature
 * (any may be NULL), dL/dlaplace, ACCUMULATES dL/dtable (float32, atomic)
 * and dL/dnet (angelo_sdf_grad_size floats, atomic).  The curvature path
 * includes the hash grid's positional derivative at the shifted stencil.
 * workspace: the forward's, read only (the backward may run more than once);
 * bwd_workspace: angelo_sdf_workspace_floats(.., 1) floats of scratch. */
int angelo_sdf_stencil_bwd(const angelo_hashgrid_layout_t *lay, int32_t active_levels,
                           const void *table, int32_t table_dtype, const angelo_sdf_net_layout *nl,
                           const void *net, const float *pos, const float *rand_dirs, int64_t n,
                           float radius, float eps, int32_t with_grad, int32_t with_laplace,
                           const float *workspace, float *bwd_workspace, const float *g_sdf,
                           const float *g_grad, const float *g_feature, int64_t gfeat_stride,
                           const float *g_laplace, float *d_table, float *d_net, void *stream);

/* ------------------------------------------------- tensor-core building block */

/* Number of CTAs of the tensor-core kernels that stopped waiting for an MMA
 * completion (bounded mbarrier waits) since the last reset; synchronous, -1
 * on a CUDA error.  A diagnostic counter: the one piece of mutable device
 * state of the library besides the allocation-free scan's workspace. */
int64_t angelo_tc_timeouts(int32_t reset);

/* ------------------------------------------------------------------- AdamW */

/* One AdamW step of a float32 parameter tensor of n elements, in place
 * (replaces torch.optim.AdamW.step for the groups systems/utils.py:314-325
 * builds): p -= lr*wd*p; m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2;
 * p -= (lr/bc1) m / (sqrt(v)/sqrt(bc2) + eps).  bias_correction1/2 =
 * 1 - beta^step, computed by the caller. */
int angelo_adamw_step(float *param, const float *grad, float *exp_avg, float *exp_avg_sq, int64_t n,
                      float lr, float beta1, float beta2, float eps, float weight_decay,
                      float bias_correction1, float bias_correction2, void *stream);
/* The same update for n_tensors tensors in one launch per 32 (host arrays of
 * device pointers, sizes and per-tensor hyper-parameters); bit-identical to
 * angelo_adamw_step on each tensor.  For the many small MLP tensors. */
int angelo_adamw_step_multi(int32_t n_tensors, float *const *params, const float *const *grads,
                            float *const *exp_avg, float *const *exp_avg_sq, const int64_t *sizes,
                            const float *lr, const float *beta1, const float *beta2,
                            const float *eps, const float *weight_decay,
                            const float *bias_correction1, const float *bias_correction2,
                            void *stream);

/* ----------------------------------------------------- weight norm and loss */

/* nn.utils.weight_norm (dim 0) of n_layers <= 8 layers at once, as VanillaMLP
 * applies it to the geometry MLP (models/network_utils.py:132-133): layer i
 * has rows[i] x cols[i] row-major v[i], g[i] (rows[i] values) and output
 * w[i] = g * v / ||v||_row.  The backward writes (not accumulates)
 * dg = (dW . v) / n and dv = (g / n) dW - (g (dW . v) / n^3) v, n = ||v||_row.
 * Pointer arrays are host arrays of device pointers. */
int angelo_weight_norm_fwd(int32_t n_layers, const int32_t *rows, const int32_t *cols,
                           const float *const *v, const float *const *g, float *const *w,
                           void *stream);
int angelo_weight_norm_bwd(int32_t n_layers, const int32_t *rows, const int32_t *cols,
                           const float *const *v, const float *const *g, const float *const *dw,
                           float *const *dv, float *const *dg, void *stream);

/* The loss the NeuS training step seeds (systems/neus.py:130-159): rgb MSE
 * over the valid rays (valid: n_rays bytes, nonzero = valid), eikonal
 * mean((||grad|| - 1)^2) over n_samples, curvature mean(|laplace|) (laplace
 * may be NULL: term 0).  out (device float[5]) = total = w_rgb rgb +
 * w_eikonal eikonal + w_curvature curvature (the curvature term only when
 * w_curvature > 0), rgb, eikonal, curvature, n_valid.  No valid ray gives a
 * NaN rgb term, as the reference's mse over an empty selection does.
 * workspace: angelo_loss_workspace_size() bytes, zeroed once before the
 * first call (the call leaves it zeroed).  Sums reduce in a fixed order.
 * The backward writes dL/d(rgb_pred), dL/d(sdf_grad) and (when d_laplace is
 * not NULL) dL/d(laplace) for dL/dtotal = *d_total, from the forward's out
 * (stats). */
int64_t angelo_loss_workspace_size(void);
int angelo_neus_loss_fwd(const float *rgb_pred, const float *rgb_true, const uint8_t *valid,
                         int64_t n_rays, const float *sdf_grad, const float *laplace,
                         int64_t n_samples, float w_rgb, float w_eikonal, float w_curvature,
                         void *workspace, float *out, void *stream);
int angelo_neus_loss_bwd(const float *rgb_pred, const float *rgb_true, const uint8_t *valid,
                         int64_t n_rays, const float *sdf_grad, const float *laplace,
                         int64_t n_samples, float w_rgb, float w_eikonal, float w_curvature,
                         const float *stats, const float *d_total, float *d_rgb, float *d_grad,
                         float *d_laplace, void *stream);

/* ----------------------------------------------------- fused radiance network */

/* Bytes of the prepared radiance-MLP buffer for a feature input of feat_dim
 * columns (the MLP input is [feature, SH4 (16), normal (3)] = feat_dim + 19
 * <= 96); -1 when unsupported. */
int64_t angelo_radiance_net_bytes(int32_t feat_dim);
/* Floats of the flat weight gradient: [dW1 (64 x 16*ceil(in/16)), dW2 (64x64),
 * dW3 (16 x 64), db1 (64), db2 (64), db3 (16)]. */
int64_t angelo_radiance_grad_size(int32_t feat_dim);
/* Effective fp32 weights of VanillaMLP(in, 3, 2 hidden ReLU layers of 64)
 * (models/texture.py:19,47) -> prepared buffer (bf16 hi/lo operands). */
int angelo_radiance_prep(int32_t feat_dim, const float *W1, const float *b1, const float *W2,
                         const float *b2, const float *W3, const float *b3, void *net,
                         void *stream);
/* The same with the operands in ANGELO_OPERAND_BF16 or ANGELO_OPERAND_FP16
 * parts; an fp16 buffer serves angelo_radiance_fwd with flags bit 2 only
 * (the backward reads bf16 operands). */
int angelo_radiance_prep_format(int32_t feat_dim, int32_t operand_format, const float *W1,
                                const float *b1, const float *W2, const float *b2,
                                const float *W3, const float *b3, void *net, void *stream);
/* VolumeRadiance / VolumeDualColor forward (models/texture.py:23-30,50-58):
 * rgb = sigmoid(MLP([feature, SH4((d+1)/2), normalize(grad)])) (+ sigmoid of
 * feature[1:4] when dual), d = rays_d[ray_idx].  flags bit 0: dual colour;
 * bit 1: the MLP in a single pass (hi parts alone) instead of three
 * products; bit 2: fp16 operands (a buffer from angelo_radiance_prep_format
 * with ANGELO_OPERAND_FP16) instead of bf16.  grad may be NULL: a network
 * without a normal input (VolumeRadiance on [feature, SH4], the learned
 * background's texture), whose W1 normal columns the caller sets to zero. */
int angelo_radiance_fwd(int32_t feat_dim, const void *net, const float *feature,
                        int64_t feat_stride, const float *grad, const int32_t *ray_idx,
                        const float *rays_d, int64_t n, int32_t flags, float *rgb, void *stream);
/* Backward: d_feature (written, n x feat_stride), d_grad (written, n x 3;
 * NULL exactly when grad is NULL), d_net (accumulated). */
int angelo_radiance_bwd(int32_t feat_dim, const void *net, const float *feature,
                        int64_t feat_stride, const float *grad, const int32_t *ray_idx,
                        const float *rays_d, int64_t n, int32_t dual, const float *g_rgb,
                        float *d_feature, float *d_grad, float *d_net, void *stream);

/* ------------------------------------------------------------ fused VanillaMLP */

/* VanillaMLP with ReLU between layers and no output activation
 * (models/network_utils.py:96-140 as the learned background's density
 * network uses it, models/geometry.py:152-177): in_dim (1..64) inputs,
 * n_hidden (1 or 2) hidden layers of 64, out_dim (1..16) outputs, on the
 * tensor cores (bf16x3 operands, fp32 accumulation).  Bytes of the prepared
 * buffer; -1 when the shape is unsupported. */
int64_t angelo_mlp_net_bytes(int32_t in_dim, int32_t n_hidden, int32_t out_dim);
/* Floats of the flat weight gradient: [dW1 (64 x 16*ceil(in_dim/16)),
 * dW2 (64 x 64, two hidden layers), dW3 (16 x 64), db1 (64), db2 (64, two
 * hidden layers), db3 (16)]; -1 when unsupported. */
int64_t angelo_mlp_grad_size(int32_t in_dim, int32_t n_hidden, int32_t out_dim);
/* fp32 weights (row-major [out][in], as nn.Linear keeps them; W2, b2 may be
 * NULL with one hidden layer) -> prepared buffer. */
int angelo_mlp_prep(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const float *W1,
                    const float *b1, const float *W2, const float *b2, const float *W3,
                    const float *b3, void *net, void *stream);
/* out[i] (out_dim columns, row stride out_stride) = MLP(x[i]) (in_dim
 * columns, row stride x_stride) for n rows (replaces the torch / tcnn
 * network call of models/network_utils.py:134-140). */
int angelo_mlp_fused_fwd(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const void *net,
                         const float *x, int64_t x_stride, int64_t n, float *out,
                         int64_t out_stride, void *stream);
/* Backward from dL/dout (g_out, row stride g_stride): writes dL/dx (d_x, row
 * stride dx_stride; may be NULL) and ACCUMULATES dL/dW into d_net
 * (angelo_mlp_grad_size floats).  The hidden activations are recomputed
 * from x; with x_rows (may be NULL), row i of the call reads x row
 * x_rows[i] (the inputs of a subset of an earlier forward's rows, without
 * copying them out). */
int angelo_mlp_fused_bwd(int32_t in_dim, int32_t n_hidden, int32_t out_dim, const void *net,
                         const float *x, int64_t x_stride, const int32_t *x_rows, int64_t n,
                         const float *g_out,
                         int64_t g_stride, float *d_x, int64_t dx_stride, float *d_net,
                         void *stream);

/* ------------------------------------------- fused background compositing */

/* The learned background's compositing in one warp per ray
 * (models/neus.py:171-177: nerfacc 0.3.3 render_weight_from_density, then
 * accumulate_along_rays of 1, the interval midpoints and the colours, and
 * the background colour blended behind): w_j = (1 - e^-tau_j)
 * e^-(tau_0 + .. + tau_{j-1}), tau_j = sigma_j (t_end - t_start);
 * opacity (n_rays), depth (n_rays), comp_rgb (n_rays x 3) = sum w rgb +
 * bg (1 - opacity).  weights and trans (per sample) are kept for the
 * backward. */
int angelo_density_composite_fwd(const int64_t *offsets, int64_t n_rays, const float *sigmas,
                                 const float *t_starts, const float *t_ends, const float *rgb,
                                 const float *bg, float *opacity, float *depth, float *comp_rgb,
                                 float *weights, float *trans, void *stream);
/* Backward from dL/dopacity, dL/ddepth, dL/dcomp_rgb (each may be NULL =
 * zero): writes dL/dsigma (per sample) and dL/drgb (per sample x 3). */
int angelo_density_composite_bwd(const int64_t *offsets, int64_t n_rays, const float *sigmas,
                                 const float *t_starts, const float *t_ends, const float *rgb,
                                 const float *bg, const float *weights, const float *trans,
                                 const float *g_opacity, const float *g_depth, const float *g_rgb,
                                 float *d_sigmas, float *d_rgb, void *stream);

/* The samples' world points (models/neus.py:222-226): midpoint
 * m = (t_start + t_end) * 0.5 and point o + d * m of ray ray_indices[j], in
 * that order of float32 operations (bit-identical to the reference's torch
 * expression); midpoints (n floats) is optional. */
int angelo_sample_points(const float *rays_o, const float *rays_d, const int32_t *ray_indices,
                         const float *t_starts, const float *t_ends, int64_t n, float *points,
                         float *midpoints, void *stream);

/* The learned background's sample points and visibility test
 * (models/neus.py:141-170), one launch each.  bg_points: the world point
 * o + d (t_start + t_end)/2 of every sample, contracted to [0,1]^3 by the
 * unbounded-sphere contraction of radius (models/geometry.py:22-28).
 * bg_visibility: per ray the number of leading samples whose transmittance
 * (sequential float32 product of 1 - alpha, alpha = 1 - exp(-exp(out0 +
 * density_bias) dt), out0 = out[j * out_stride]) is at least early_stop_eps:
 * nerfacc's visibility test keeps that prefix of each ray.  bg_compact:
 * those samples (their ray index, t, point, out_dim outputs and their row in
 * the inputs) at kept_offsets, the exclusive scan of kept. */
int angelo_bg_points(const float *rays_o, const float *rays_d, const int32_t *ray_indices,
                     const float *t_starts, const float *t_ends, int64_t n, float radius,
                     float *points, void *stream);
int angelo_bg_visibility(const float *out, int64_t out_stride, float density_bias,
                         const float *t_starts, const float *t_ends, const int64_t *offsets,
                         int64_t n_rays, float early_stop_eps, int32_t *kept, void *stream);
int angelo_bg_compact(const int64_t *offsets, const int32_t *kept, const int64_t *kept_offsets,
                      int64_t n_rays, const int32_t *ray_indices, const float *t_starts,
                      const float *t_ends, const float *points, const float *out, int32_t out_dim,
                      int32_t *ray_indices_k, float *t_starts_k, float *t_ends_k, float *points_k,
                      float *out_k, int32_t *rows_k, void *stream);

/* ------------------------------------------------------------------ serving */

/* The resident field a server renders: device pointers owned by the caller
 * and left unchanged while the server lives (hash table; SDF MLP prepared by
 * angelo_sdf_prep; radiance MLP prepared by angelo_radiance_prep; occupancy
 * bits).  This is the trained NeuSModel the reference's eval path renders
 * (models/neus.py:285-293). */
typedef struct {
    angelo_hashgrid_layout_t lay;
    int32_t active_levels;
    const void *table;
    int32_t table_dtype;
    angelo_sdf_net_layout sdf_layout;
    const void *sdf_net;
    float radius;
    float eps;                 /* finite-difference step of the normal */
    int32_t feat_dim;          /* radiance feature width = sdf out_dim + 3 */
    const void *rad_net;
    int32_t rad_flags;         /* angelo_radiance_fwd flags (bit 0: dual colour) */
    const float *variance;     /* device float: inv_s = exp(10 variance) */
    float cos_anneal_ratio;
    const float *background;   /* device float[3], blended behind each ray */
    angelo_grid_t grid;        /* occupancy grid of the march */
    float render_step;
    int32_t max_steps;
    float near_plane;          /* near / far planes; both < 0: the scene box */
    float far_plane;           /* [-radius, radius]^3 (one < 0: that plane unset) */
} angelo_serve_field;

/* sizeof(angelo_serve_field), for bindings that mirror the struct. */
int64_t angelo_serve_field_bytes(void);

typedef struct angelo_server angelo_server;

/* A server of fixed-shape buckets: rays_per_bucket rays with a capacity of
 * samples_per_ray samples each, points_per_bucket SDF points.  Allocates the
 * bucket's device buffers, runs one bucket to set the kernels up and, with
 * use_graph, captures the render bucket as a CUDA graph (thread-local
 * capture on a stream of its own).  Synchronous. */
int angelo_serve_create(const angelo_serve_field *field, int64_t rays_per_bucket,
                        int32_t samples_per_ray, int64_t points_per_bucket, int32_t use_graph,
                        angelo_server **out);
/* Render n rays (device, n x 3 origins and directions) in buckets on stream:
 * rgb (n x 3, background blended), opacity (n), depth (n), as
 * NeuSModel.forward in eval mode gives comp_rgb_full, opacity and depth.
 * A bucket whose samples overflow its capacity is rendered again at its
 * exact size; *overflows (may be NULL) counts them.  Returns after the
 * outputs are written (one stream synchronisation per call).  A server's
 * bucket buffers serve one call at a time: calls on one server from several
 * threads or streams race (create one server per stream). */
int angelo_serve_render(angelo_server *srv, const float *rays_o, const float *rays_d, int64_t n,
                        float *rgb, float *opacity, float *depth, int64_t *overflows, void *stream);
/* SDF at n device points (VolumeSDF.forward_level, the isosurface lattice of
 * models/geometry.py:84-92), points_per_bucket at a time; asynchronous. */
int angelo_serve_sdf(angelo_server *srv, const float *points, int64_t n, float *sdf, void *stream);
/* Waits for the device and frees the server's buffers and graph. */
int angelo_serve_destroy(angelo_server *srv);

/* ------------------------------------------------------------ fused compositing */

/* NeuSModel.get_alpha + render_weight_from_alpha + accumulate_along_rays + the
 * background blend (models/neus.py:117-139,234-248,273-277), one warp per ray:
 * alpha from sdf / normalize(grad) / ray direction / interval with inv_s =
 * clip(exp(10*variance)) read on the device (fp64 when inv_s > fp64_gate),
 * log-space transmittance by a warp prefix sum, weights zero once
 * T < early_stop_eps; per-ray opacity, depth, comp_rgb, comp_normal
 * (normalised, zero where opacity <= 0.1), comp_rgb_full = comp_rgb +
 * bg*(1-opacity).  acc_normal (unnormalised sum), weights and trans (per
 * sample) are kept for the backward; alpha may be NULL. */
int angelo_composite_fwd(const int64_t *offsets, int64_t n_rays, const float *sdf,
                         const float *grad, const float *t_starts, const float *t_ends,
                         const float *rays_d, const float *rgb, const float *variance,
                         float cos_anneal_ratio, const float *bg, float early_stop_eps,
                         float fp64_gate, float *opacity, float *depth, float *comp_rgb,
                         float *comp_normal, float *comp_rgb_full, float *acc_normal,
                         float *weights, float *trans, float *alpha, void *stream);
/* Backward by a reverse affine warp scan R_{j-1} = (1-a_j) R_j + g_j a_j,
 * dL/dalpha_j = T_j (g_j - R_j): writes d_sdf, d_grad (n x 3), d_rgb (n x 3)
 * and ACCUMULATES d_variance (1 float).  Any output gradient may be NULL. */
int angelo_composite_bwd(const int64_t *offsets, int64_t n_rays, const float *sdf,
                         const float *grad, const float *t_starts, const float *t_ends,
                         const float *rays_d, const float *rgb, const float *variance,
                         float cos_anneal_ratio, const float *bg, float early_stop_eps,
                         float fp64_gate, const float *opacity, const float *acc_normal,
                         const float *weights, const float *trans, const float *g_opacity,
                         const float *g_depth, const float *g_comp_rgb,
                         const float *g_comp_normal, const float *g_comp_rgb_full, float *d_sdf,
                         float *d_grad, float *d_rgb, float *d_variance, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ANGELO_GB_H */
