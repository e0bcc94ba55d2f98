/*
 * mplicits.h -- C ABI of libmplicits.so, the GB300 (sm_103a) kernels for the
 * M-plicits nested sine-MLP hot path: f = f0 + f1 + f2, each residual level
 * evaluated only inside the delta-band of the previous partial sum, band-culled
 * marching cubes, sphere tracing and analytic normals.
 *
 * Conventions
 *  - Every entry point returns an int status (MPL_OK == 0); nothing throws.
 *  - All pointers named *_dev, and every array argument unless stated
 *    otherwise, are device pointers owned by the caller.  The library never
 *    allocates device memory inside a call (the one exception is the setup
 *    call mpl_scene_create): scratch space is caller-provided and sized by
 *    the matching *_bytes query.
 *  - `stream` is a cudaStream_t passed as void*; every launch is
 *    stream-ordered, and no call synchronises the host unless its comment
 *    says so.
 *  - A SIREN level is the network of i3d/model.py:76-103: n_layers nn.Linear
 *    layers, dims[l] -> dims[l+1], each but the last followed by
 *    sin(omega[l] * .).  Weights are the nn.Linear tensors, [out, in]
 *    row-major float32.
 */
#ifndef MPLICITS_H_
#define MPLICITS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPL_ABI_VERSION 1
#define MPL_MAX_LAYERS 8

/* status codes */
enum {
  MPL_OK = 0,
  MPL_ERR_INVALID_ARG = 1,   /* null pointer, bad size, misaligned buffer     */
  MPL_ERR_UNSUPPORTED = 2,   /* shape or mode this build has no kernel for    */
  MPL_ERR_CAPACITY = 3,      /* an output list or workspace is too small      */
  MPL_ERR_DEVICE_TIMEOUT = 4,/* a bounded device-side wait gave up            */
  MPL_ERR_CUDA = 5,          /* a CUDA runtime call failed (see last error)   */
  MPL_ERR_NO_DEVICE = 6      /* no sm_103 device is current                   */
};

/* arithmetic of the hidden-layer GEMMs */
enum {
  MPL_FP32 = 0, /* plain form: FP32 SIMT FMAs, accurate sinf               */
  MPL_BF16 = 1, /* tcgen05 BF16 MMAs, FP32 accumulate in TMEM, FP32 layer 0 */
  MPL_F16 = 2   /* the same kernels with FP16 operands: same speed, 8x finer
                   rounding of the sine activations (all within [-1, 1])   */
};

/* how a level's output is stored */
enum {
  MPL_STORE = 0,     /* S[p]  = f(x_p)                                      */
  MPL_ACCUMULATE = 1 /* S[p] += f(x_p)   (i3d/meshing.py:231 sdf_base[idx] +=) */
};

/* where the points come from */
enum {
  MPL_POINTS_XYZ = 0, /* explicit float32 [n, 3] coordinates               */
  MPL_POINTS_GRID = 1 /* grid point p of gen_mc_coordinate_grid, generated
                         in-kernel with the reference's float32 formula     */
};

/* Topology of one level. */
typedef struct MplNet {
  int32_t n_layers;                  /* nn.Linear layers, 2..MPL_MAX_LAYERS   */
  int32_t dims[MPL_MAX_LAYERS + 1];  /* dims[0] == 3, dims[n_layers] == 1,
                                        hidden widths <= 256                   */
  float omega[MPL_MAX_LAYERS];       /* sine frequency after layer l          */
} MplNet;

/* A point set.  For MPL_POINTS_GRID point p (0 <= p < N^3) is row p of
 * gen_mc_coordinate_grid(N, voxel_size) (i3d/meshing.py:42-63), including
 * the float32 true-division shear of its x and y columns.  offset[c] is the
 * constant added to column c (the reference adds voxel_origin[2], [1], [0]).*/
typedef struct MplPoints {
  int32_t kind;        /* MPL_POINTS_XYZ or MPL_POINTS_GRID                 */
  int32_t grid_n;      /* N (GRID)                                          */
  float voxel_size;    /* float32 voxel size (GRID)                          */
  float offset[3];     /* per-column offset (GRID)                           */
  const float* xyz;    /* [n, 3] float32 (XYZ)                               */
} MplPoints;

/* Fused band compaction: after a level stores S[p], p is appended to
 * out_index when lower <= |S[p]| < delta (float32 compares; lower = 0 gives
 * the reference's |S| < delta of i3d/meshing.py:223).  *count_dev is reset
 * to 0 by the call.  Entries past `capacity` are dropped but still counted,
 * so *count_dev > capacity reports an overflow.  The order of out_index is
 * unspecified; its set is exact. */
typedef struct MplBand {
  float delta;
  int32_t* out_index;  /* device [capacity]                                  */
  int32_t* count_dev;  /* device int32 scalar                                */
  int64_t capacity;
  float lower;         /* keep only |S| >= lower (0: no lower bound)         */
} MplBand;

/* A pinhole camera: look-at eye/target/up, vertical field of view, image
 * size.  Pixel (i, j) has NDC x = 2i/W - 1 and y = 1 - 2j/H, as the
 * reference's ray tests (renderer/cuda/tests/tests.cu:73-87). */
typedef struct MplCamera {
  float eye[3];
  float target[3];
  float up[3];
  float fov_y_deg;
  int32_t width;
  int32_t height;
} MplCamera;

/* ---- weights ------------------------------------------------------------ */

/* Bytes of the packed device image of one level (FP32 and BF16 forms). */
int mpl_net_packed_bytes(const MplNet* net, int64_t* bytes);

/* Packs a level's nn.Linear tensors (device pointers, weights[l] is
 * [dims[l+1], dims[l]], biases[l] is [dims[l+1]]) into `packed_dev`
 * (>= mpl_net_packed_bytes, 256-byte aligned).  Replaces the per-layer
 * tensors the reference's LayerGemm holds (renderer/cuda/gemms.cu:5-100). */
int mpl_net_pack(const MplNet* net, const float* const* weights_dev,
                 const float* const* biases_dev, void* packed_dev, void* stream);

/* ---- level evaluation (i3d/model.py:107-129; i3d/meshing.py:212-236) ---- */

/* Evaluates one level on points q = 0..n-1, where the point is
 * p = index ? index[q] : q, and stores or accumulates f(x_p) into S[p].
 * If n_dev is non-null, the point count is min(*n_dev, n) read on the
 * device (so a band list produced by a previous call can be consumed
 * without a host round trip).  `band` (nullable) appends the points of
 * the next delta-band.  precision: MPL_FP32 or MPL_BF16. */
int mpl_level_forward(const MplNet* net, const void* packed_dev, const MplPoints* points,
                      const int32_t* index_dev, const int32_t* n_dev, int64_t n,
                      float* S_dev, int32_t store_mode, const MplBand* band,
                      int32_t precision, void* stream);

/* Writes the float32 coordinates [n, 3] of grid points p = index ? index[q]
 * : q (points->kind must be MPL_POINTS_GRID): the columns 0..2 of
 * gen_mc_coordinate_grid (i3d/meshing.py:11-69), bit for bit. */
int mpl_grid_points(const MplPoints* points, const int32_t* index_dev, int64_t n,
                    float* xyz_dev, void* stream);

/* As mpl_level_forward, and also stores (or accumulates) the input gradient
 * df/dx of every point into G[3p .. 3p+2] in one launch, by forward-mode
 * differentiation through the fused level.  Replaces the autograd gradient
 * of i3d/diff_operators.py:259-265 (normals, eikonal term) and the
 * reference renderer's per-coordinate Normals GEMM chains
 * (renderer/cuda/gemms.cu:206-337, kernels.cu:277-313). */
int mpl_level_gradient(const MplNet* net, const void* packed_dev, const MplPoints* points,
                       const int32_t* index_dev, const int32_t* n_dev, int64_t n, float* S_dev,
                       float* G_dev, int32_t store_mode, const MplBand* band, int32_t precision,
                       void* stream);

/* ---- band compaction (i3d/meshing.py:222-231) --------------------------- */

/* Appends q's point p = index ? index[q] : q for q < n (or < *n_dev) with
 * band->lower <= |S[p]| < band->delta to band->out_index. */
int mpl_band_compact(const float* S_dev, const int32_t* index_dev, const int32_t* n_dev,
                     int64_t n, const MplBand* band, void* stream);

/* max_j |S[j]| over S[0 .. n) into *out_dev (device float; 0 for n = 0, NaN
 * if any S[j] is NaN), stream-ordered, no host sync.  Replaces the per-chunk
 * `float(s.abs().max())` of adaptive_deltas (reconstruct.py:28-31), which
 * reads every chunk's maximum back to the host. */
int mpl_abs_max(const float* S_dev, int64_t n, float* out_dev, void* stream);

/* ---- marching cubes (i3d/meshing.py:267-313; scikit-image's
 *      marching_cubes, replaced by a table derived in this project) ------- */

/* Workspace bytes for an N^3 volume. */
int mpl_mc_workspace_bytes(int64_t N, int64_t* bytes);

/* Classifies every cell of the C-order N^3 volume S and writes
 * counts_dev[0] = vertices, counts_dev[1] = triangles (int64). */
int mpl_mc_count(const float* S_dev, int64_t N, float iso, void* workspace_dev,
                 int64_t* counts_dev, void* stream);

/* Emits the mesh counted by the preceding mpl_mc_count on the same
 * workspace.  Vertices are ordered by (lower grid point, axis) of their edge,
 * faces by cell then case-table order.  verts/normals [V,3] f32, values [V]
 * f32 (nullable), faces [F,3] int32.  Coordinates are
 * ((float)index + t) * voxel_size + origin[axis]. */
int mpl_mc_emit(const float* S_dev, int64_t N, float iso, float voxel_size,
                const float* origin_host, const void* workspace_dev, float* verts_dev,
                float* normals_dev, float* values_dev, int32_t* faces_dev, int64_t max_verts,
                int64_t max_tris, void* stream);

/* Marching cubes in one call that allocates nothing.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory, such
 * as a real-time frame loop that must not pay the device-wide
 * synchronisation of cudaMalloc/cudaFree, or a host program that can only
 * pass buffers it registered itself.  The count/prefix workspace lives in a
 * fixed device array inside the library (1.5 MiB, held on every GPU that
 * loads the library until exit), so N is limited to 256; a larger N returns
 * MPL_ERR_CAPACITY.  The first call on each device does one-time set-up
 * (it looks up the array's device address and uploads the case tables);
 * make that first call before any stream capture.  First calls from several
 * host threads at once are safe: the set-up is serialised and done once.
 * Calls that overlap on the GPU share the array and race: order them on one
 * stream.  Output as mpl_mc_emit, with
 * counts_dev[0], [1] = the full vertex and triangle counts (int64); output
 * beyond max_verts / max_tris is dropped, so counts above the capacities
 * mean the mesh was cut short. */
int mpl_mc_noalloc(const float* S_dev, int64_t N, float iso, float voxel_size,
                   const float* origin_host, float* verts_dev, float* normals_dev,
                   float* values_dev, int32_t* faces_dev, int64_t max_verts, int64_t max_tris,
                   int64_t* counts_dev, void* stream);

/* ---- sphere tracing (renderer/cuda/kernels.cu:315-487, state.cu:848-880) */

/* Generates one ray per pixel into origins/dirs [W*H, 3], moves every origin
 * outside the bounding sphere of `radius` onto it (kernels.cu:454-477), sets
 * state[r] = 0 (marching) or 2 (misses the sphere) and writes the marching
 * rays to active[0 .. *count).  Replaces InitializeRays_kernel
 * (kernels.cu:400-487). */
int mpl_trace_init(const MplCamera* camera, float radius, float* origins_dev, float* dirs_dev,
                   int32_t* state_dev, int32_t* active_dev, int32_t* count_dev, void* stream);

/* One marching step over the rays active[0 .. min(*count, n_max)), whose
 * distance S[r] the level launches have just produced: |S| < eps marks a hit
 * (state 1, appended to hit_out / *hit_count, which the caller zeroes once
 * per frame); otherwise origins += dirs * S, and a ray leaving the sphere
 * outwards is a miss (state 2); with last_step set the remaining rays get
 * state 3.  Marching rays go to active_out / *count_out (reset by the call).
 * Replaces IterateSphereTracing_kernel (kernels.cu:315-398). */
int mpl_trace_step(const float* S_dev, const int32_t* active_dev, const int32_t* count_dev,
                   int64_t n_max, float* origins_dev, const float* dirs_dev, int32_t* state_dev,
                   float eps, float radius, int32_t last_step, int32_t* active_out_dev,
                   int32_t* count_out_dev, int32_t* hit_out_dev, int32_t* hit_count_dev,
                   int64_t capacity, void* stream);

/* Every remaining marching step of the rays active[0 .. min(*count, n_max))
 * in one launch, on the tensor cores (BF16 or FP16 operands, `precision`):
 * per step the `levels` nets (identical hidden widths) are evaluated at the
 * rays' positions, level l > 0 added only for rays with |partial sum| <
 * deltas[l - 1] (the band lists of the level launches), then each ray takes
 * the step of mpl_trace_step (S written, hits appended to hit_out /
 * *hit_count); with last_is_final set the last of the `steps` steps ends the
 * budget (state 3).  Gives every ray the result of `steps` rounds of level
 * launches + mpl_trace_step; a launch keeps one CTA per 128 rays, so it pays
 * off once few rays are left.  Replaces the tail of the reference's per-level
 * phases (state.cu:848-880) over IterateSphereTracing_kernel
 * (kernels.cu:315-398).  MPL_ERR_UNSUPPORTED for widths other than 128/256
 * or when the levels' constants exceed shared memory. */
int mpl_trace_march(const MplNet* nets, const void* const* packed_dev, int32_t levels,
                    const float* deltas, const int32_t* active_dev, const int32_t* count_dev,
                    int64_t n_max, float* origins_dev, const float* dirs_dev, int32_t* state_dev,
                    float* S_dev, float eps, float radius, int32_t steps, int32_t last_is_final,
                    int32_t* hit_out_dev, int32_t* hit_count_dev, int64_t capacity,
                    int32_t precision, void* stream);

/* Shades every pixel into RGBA8 (little-endian R in the low byte): hits
 * inside [-1,1]^3 with Phong (mode 1) or |normal| colours (mode 0) from the
 * gradients G [P, 3], everything else white.  Replaces Shade_kernel
 * (kernels.cu:122-275) writing a headless buffer instead of a GL PBO. */
int mpl_trace_shade(const float* origins_dev, const float* dirs_dev, const float* G_dev,
                    const int32_t* state_dev, int64_t P, int32_t mode, uint32_t* image_dev,
                    void* stream);

/* ---- training (i3d/loss_functions.py:327-394,
 *      experiment_scripts/train_sdf_on_neighborhood_fine.py:197-262) ------- */

/* Floats of the pre-activation scratch of mpl_train_forward for n points:
 * (hidden GEMMs + 1) * n * 4 * padded width. */
int mpl_train_scratch_floats(const MplNet* net, int64_t n, int64_t* floats);

/* Plain-form forward of a trainable level on xyz [n, 3]: S [n], G [n, 3]
 * (df/dx) and the pre-activations of every layer for the backward. */
int mpl_train_forward(const MplNet* net, const void* packed_dev, const float* xyz_dev, int64_t n,
                      float* S_dev, float* G_dev, float* pre_dev, void* stream);

/* Loss of a training step. */
enum {
  MPL_LOSS_RESIDUAL = 0, /* loss_add_detail(_fine), i3d/loss_functions.py:263-394:
                            weight = {sdf, normal, eikonal, -}; S and G include
                            the frozen levels' sums; gt == -1 marks points
                            without SDF and normal supervision               */
  MPL_LOSS_TRUE_SDF = 1  /* true_sdf, i3d/loss_functions.py:123-163 (the coarse
                            trainer): weight = {sdf on surface, sdf off surface,
                            normal, eikonal}; gt == 0 marks surface points     */
};

typedef struct MplLoss {
  int32_t kind;
  float weight[4];
} MplLoss;

/* A trainer's loss on n points with S = f + f_frozen and G = g + g_frozen
 * (f_frozen, g_frozen nullable): the per-term sums over the points into
 * loss_sums[4] (divide by n and weight as the reference does; the residual
 * loss has three terms, the fourth sum is 0) and the derivative seeds
 * seeds [n, 4] = (dL/df, dL/dG) of the weighted mean loss. */
int mpl_train_loss(int64_t n, const float* f_dev, const float* g_dev, const float* f_frozen_dev,
                   const float* g_frozen_dev, const float* gt_sdf_dev, const float* gt_normals_dev,
                   const MplLoss* loss, float* seeds_dev, float* loss_sums_dev, void* stream);

/* Weight gradients of a loss given its seeds on (f, df/dx) of every point:
 * the backward through the level's forward-mode graph (double backward of
 * the input gradient included).  dW[l] / db[l] are device buffers of the
 * padded shapes ([WP][3] for layer 0, [WP][WP] hidden, [WP] output; bias
 * [WP], output bias [1]); the call ADDS into them.  `da` is scratch of the
 * same size as the pre-activations.  Replaces autograd's backward of
 * torch.autograd.grad(..., create_graph=True) in the reference trainers. */
int mpl_train_backward(const MplNet* net, const void* packed_dev, const float* xyz_dev, int64_t n,
                       const float* pre_dev, const float* seeds_dev, float* da_dev,
                       float* const* dW_dev, float* const* db_dev, void* stream);

/* Bytes of the device scratch of mpl_train_tc_step for n points: the BF16
 * activation and adjoint tiles of every layer, 2 * (hidden GEMMs + 1) *
 * rows * padded width * 2 with rows = 4 * n rounded up to 128. */
int mpl_train_tc_scratch_bytes(const MplNet* net, int64_t n, int64_t* bytes);

/* The training step of one level on the tensor cores (BF16 operands, FP32
 * accumulation, FP32 master weights outside): forward in forward mode, the
 * loss with S = f + f_frozen and G = df/dx + g_frozen (as mpl_train_loss:
 * sums into loss_sums[4], seeds [n, 4] written, 16-byte aligned), the
 * backward through the forward-mode graph (double backward included) and
 * every weight gradient, ADDED into the padded buffers dW[l] / db[l] of
 * mpl_train_backward.  Replaces the reference trainers' forward, loss and
 * loss.backward() (experiment_scripts/train_sdf_on_neighborhood_fine.py:
 * 247-250 with i3d/loss_functions.py:347-394; the coarse trainer with
 * true_sdf).  Levels with 1 or 2 hidden GEMMs of padded width 128 or 256. */
int mpl_train_tc_step(const MplNet* net, const void* packed_dev, const float* xyz_dev, int64_t n,
                      const float* f_frozen_dev, const float* g_frozen_dev,
                      const float* gt_sdf_dev, const float* gt_normals_dev, const MplLoss* loss,
                      void* scratch_dev, int64_t scratch_bytes, float* seeds_dev,
                      float* loss_sums_dev, float* const* dW_dev, float* const* db_dev,
                      void* stream);

/* Flags of mpl_train_batch. */
#define MPL_BATCH_NEIGH_DELTA 1 /* offset scale from the last column (use_neigh_delta) */
#define MPL_BATCH_DITHER 2      /* append the dithered rows (dithering_sampling)      */

/* The residual trainers' batch, create_training_data_on_neighborhood
 * (experiment_scripts/utils.py:92-169): from n of the n_vertices rows of
 * `vertices` (row_floats >= 6 floats each: xyz, normal, [neighbourhood
 * delta]) it writes n surface rows (sdf 0), n rows offset along the normal
 * by d * u_z (sdf d * u_z, d = the row's delta or delta_eps) and, with
 * MPL_BATCH_DITHER, n rows at x + delta * u + delta / 2 * normal (sdf -1):
 * pts [2n or 3n, 3], normals [same, 3], sdf [same].  sample_index [n] (the
 * reference's randperm prefix) and uniforms [n, 3] (its torch.rand draw) are
 * nullable; when null they come from a counter-based generator keyed by
 * `seed`, indices then drawn with replacement.  n <= n_vertices.  An index
 * outside [0, n_vertices) zeroes its rows and sets MPL_ERR_INVALID_ARG in the
 * device status word. */
int mpl_train_batch(const float* vertices_dev, int64_t n_vertices, int32_t row_floats,
                    const int64_t* sample_index_dev, const float* uniforms_dev, int64_t n,
                    float delta, float delta_eps, int32_t flags, uint64_t seed, float* pts_dev,
                    float* normals_dev, float* sdf_dev, void* stream);

/* One torch.optim.Adam step (no weight decay) over `count` FP32 tensors. */
int mpl_adam_step(int32_t count, float* const* params_dev, const float* const* grads_dev,
                  float* const* exp_avg_dev, float* const* exp_avg_sq_dev, const int64_t* numel,
                  float lr, float beta1, float beta2, float eps, int64_t step, void* stream);

/* ---- triangle scene and the tubular-neighbourhood deltas ----------------- */
/* Stand-in for the open3d RaycastingScene the neighbourhood trainers build
 * (experiment_scripts/train_sdf_on_neighborhood.py:145-146) and query with
 * compute_distance: a uniform grid over the mesh (cell side `cell`, or twice
 * the mean edge length when cell == 0) whose cells list the triangles that
 * overlap them.  Setup, not the hot path: mpl_scene_create synchronises
 * `stream` and allocates the scene's device memory itself (the one exception
 * to the caller-owned-memory rule; mpl_scene_destroy waits for the device's
 * queued work and frees it).  mpl_scene_destroy synchronises the whole
 * device (cudaDeviceSynchronize: every stream of the process is waited for),
 * so it must not run while any thread is capturing a CUDA graph, whose
 * capture that synchronisation would invalidate.  positions
 * [n_positions, 3] float32, faces [n_faces, 3] int32; a face index outside
 * [0, n_positions) gives MPL_ERR_INVALID_ARG.  The scene copies the corners:
 * the inputs may be freed after the call.  Queries must be made with the
 * scene's device current (else MPL_ERR_INVALID_ARG). */
typedef struct MplScene MplScene;
int mpl_scene_create(const float* positions_dev, int64_t n_positions, const int32_t* faces_dev,
                     int64_t n_faces, float cell, MplScene** scene, void* stream);
int mpl_scene_destroy(MplScene* scene);
/* grid geometry (host values; any pointer may be null) */
int mpl_scene_info(const MplScene* scene, float* lo3, float* cell, int32_t* dims3,
                   int64_t* n_refs);
/* Unsigned distance from each point [n, 3] to the nearest triangle
 * (RaycastingScene.compute_distance), float32, exact for the float32
 * closest-point computation stated in the source; NaN for a point with a
 * non-finite coordinate. */
int mpl_scene_compute_distance(const MplScene* scene, const float* points_dev, int64_t n,
                               float* distances_dev, void* stream);
/* calc_deltas (experiment_scripts/utils.py:46-89): out [n_vertices, cols + 1]
 * is the input rows (cols >= 6: xyz, normal, ...) with the normal
 * normalised and the bisected neighbourhood radius appended.  step0 is the
 * first step, max_delta / n_iters as the reference computes it (utils.py:57:
 * in double for a Python float max_delta, in float32 for a float32 tensor,
 * then rounded to float32); the loop runs while max(delta) < max_delta,
 * n_iters times at most (the reference uses eps 2e-4).  scratch
 * is sized by mpl_calc_deltas_scratch_bytes (256-byte aligned).
 * iterations_dev (nullable, device int32) receives the number of
 * iterations run.  Results equal the reference loop over an exact
 * nearest-triangle distance bit for bit. */
int mpl_calc_deltas_scratch_bytes(int64_t n_vertices, int32_t n_iters, int64_t* bytes);
int mpl_calc_deltas(const MplScene* scene, const float* vertices_dev, int64_t n_vertices,
                    int32_t cols, float max_delta, float step0, int32_t n_iters, float eps,
                    void* scratch_dev, float* out_dev, int32_t* iterations_dev, void* stream);

/* ---- batched evaluation of many levels of many models ------------------- */
/* No single reference entry point: this replaces the reference's one launch
 * chain per model and per level (renderer/cuda/gemms.cu:5-192 NeuralImplicit,
 * and the per-level loop of i3d/meshing.py:212-236) by one persistent launch
 * per width group of entries (see mpl_batch_run).  Entries are levels with 1
 * or 2 hidden GEMMs of width
 * <= 256 (padded widths 64/128/256 may mix); each runs on its own point list
 * (points + optional index list, count optionally on the device) and stores
 * or accumulates into its own S.  Tensor-core operands only (MPL_BF16 or
 * MPL_F16); results equal mpl_level_forward of the same entry bit for bit
 * under the same epilogue unit width. */
#define MPL_BATCH_MAX_ENTRIES 1024

typedef struct {
  MplNet net;
  const void* packed_dev; /* mpl_net_pack image, 256-byte aligned */
  MplPoints points;
  const int32_t* index_dev; /* nullable: point q is points[index[q]]  */
  const int32_t* n_dev;     /* nullable: device count, min(n, *n_dev)  */
  int64_t n;
  float* S_dev;
  int32_t store_mode;
  int32_t reserved;
} MplBatchEntry;

typedef struct {
  void* workspace_dev; /* the device entry table (entries grouped by width) */
  int32_t count;
  int32_t precision;
  int32_t width_count[3]; /* entries of padded width 64, 128, 256, in table order */
  int32_t reserved;
} MplBatchPlan;

typedef struct {
  int32_t epilogue_unit;   /* 16 or 32 features per epilogue warp (0: 32)   */
  int32_t stages;          /* weight-ring depth of the one-tile pipeline,
                              2 or 3 (0: 3); the two-tile pipeline takes the
                              level kernel's ring per width (0 only)       */
  int32_t ctas;            /* persistent CTAs (0: one per SM)              */
  int32_t tiles_in_flight; /* 2: two tiles per CTA with first-layer warps,
                              one launch per width present (unit 32 only);
                              1: one tile, first layer in the epilogue
                              warps, one launch (0: 2)                     */
} MplBatchConfig;

/* Bytes of the device workspace that holds a plan of `count` entries. */
int mpl_batch_workspace_bytes(int32_t count, int64_t* bytes);
/* Validates the entries and writes the device entry table into `workspace`
 * (256-byte aligned).  Synchronises `stream` (the host table is released on
 * return); call it outside stream capture.  Device pointers in the entries
 * must stay valid while the plan is used. */
int mpl_batch_prepare(const MplBatchEntry* entries, int32_t count, int32_t precision,
                      void* workspace_dev, int64_t workspace_bytes, MplBatchPlan* plan,
                      void* stream);
/* The plan's tiles in persistent launches: with two tiles in flight (the
 * default) a tile-prefix kernel and one batched kernel per width group
 * present, in stream order; with one tile, one launch over every entry.  No
 * host sync, so it can be captured in a CUDA graph (device counts are read by
 * every replay).  config nullable (defaults). */
int mpl_batch_run(const MplBatchPlan* plan, const MplBatchConfig* config, void* stream);
/* Times every configuration (tiles in flight x epilogue unit x weight-ring
 * depth) on the plan itself, `repeats` runs each after a warm-up run, and
 * returns the fastest (minimum time) in *best and *best_ms.  Synchronises; the entries' outputs
 * afterwards hold the result of repeated runs (re-initialise S of
 * MPL_ACCUMULATE entries before the real run). */
int mpl_batch_autotune(const MplBatchPlan* plan, int32_t repeats, MplBatchConfig* best,
                       float* best_ms, void* stream);

/* ---- tuning ------------------------------------------------------------- */

/* Process-wide kernel options (read at each launch). */
enum {
  MPL_OPT_BF16_EPILOGUE_UNIT = 1, /* features per epilogue warp and 64-wide chunk of
                                     the tensor-core level kernels and the tracing
                                     tail: 32 (8 epilogue warps, default) or 16
                                     (16 warps); the output dot's partial sums
                                     follow the unit, so roundings differ        */
  MPL_OPT_TC_TILES_IN_FLIGHT = 2, /* tiles per CTA of the tensor-core level kernel:
                                     2 (default; GEMMs of one tile overlap the
                                     epilogue of the other, results identical) or
                                     1 (single-tile kernel)                      */
  MPL_OPT_TC_GRAD_REVERSE = 3,    /* input gradient on the tensor cores: 1
                                     (default) a backward sweep over each tile of
                                     128 points (levels with one or two hidden
                                     GEMMs), 0 forward-mode tangent rows (4 rows
                                     per point); values equal, roundings differ  */
  MPL_OPT_TC_LAYER0_WARPS = 4     /* first layer of the two-tile kernel: 8
                                     (default) or 4 warps of its own, handing the
                                     first GEMM its A operand chunk by chunk, or 0
                                     (computed in the epilogue's last drain of the
                                     previous tile); results identical           */
};
int mpl_set_option(int32_t option, int64_t value);
int mpl_get_option(int32_t option, int64_t* value);

/* ---- diagnostics -------------------------------------------------------- */

const char* mpl_status_string(int status);
/* Synchronises the device, then reads and clears the device status word that
 * bounded device-side waits set when they give up (MPL_ERR_DEVICE_TIMEOUT);
 * *status_out is MPL_OK when no wait gave up. */
int mpl_device_status(int32_t* status_out);
/* Exercises the bounded-wait contract.  No counterpart in the reference: its
 * kernels have no device-side waits and it reports errors through CUDA's own
 * status (CUDA_CHECK_THROW, renderer/cuda/tools.cu:9-37).  One CTA runs the kernels' wait routine on
 * mbarriers that nothing arrives at: warp 0 with limit_ns (1 ms .. 2 s) must
 * give up and record MPL_ERR_DEVICE_TIMEOUT, warp 1 with the kernels' own
 * limit must leave through the abort flag warp 0 raised.  result_dev [4]
 * int64: whether each warp's wait succeeded, and the nanoseconds each
 * waited.  No copy or MMA is in flight, so the context stays usable. */
int mpl_wait_selftest(int64_t limit_ns, int64_t* result_dev, void* stream);
/* cudaError_t of the most recent failed CUDA call in this thread. */
int mpl_last_cuda_error(void);
int mpl_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MPLICITS_H_ */
