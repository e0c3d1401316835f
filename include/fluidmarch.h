/* fluidmarch.h -- C ABI of the GB300 SPH ray marcher (libfluidmarch.so).
 *
 * Drop-in for the reference's CPU ray marcher (Fruup/bachelor-thesis):
 *   class RayMarcher  src/app/AdvancedRenderer/RayMarcher.h:28-77
 *     RayMarcher()    RayMarcher.cpp:66-69   -> fm_create
 *     Prepare(...)    RayMarcher.cpp:76-100  -> fm_scene_create + fm_march arguments
 *     Start()         RayMarcher.cpp:102-112 -> fm_march (asynchronous on a CUDA stream)
 *     IsDone()        RayMarcher.h:44        -> fm_query
 *     Exit()          RayMarcher.cpp:71-74   -> fm_sync / fm_destroy
 *   class Frame       src/app/Dataset.h:37-65 (search build, AABB, density grid,
 *                     Dataset.cpp:9-165)     -> fm_scene_create
 *   Frame::QueryDensityGrid Dataset.cpp:26-47 -> fm_scene_download (cell of each particle)
 *
 * All entry points are plain C: opaque handles, POD structs, int status.
 * Matrices are float[16] in glm's column-major layout (m[col*4 + row]).
 * Pointers are host or device memory as the FM_MEM_* argument says; host
 * pointers are staged through device buffers the context owns.
 * No entry point falls back to a CPU path: without a usable CUDA device every
 * call that needs one returns FM_ERR_CUDA.
 *
 * Threads: a context, its scenes, batches, proposals and trainers are used by
 * one host thread at a time (the reference drives its marcher from the render
 * thread); separate contexts are independent.  A particle-file series
 * (fm_dataset_*) may be read from several threads at once.
 *
 * Streams: a call's device work goes to the stream it is given (NULL: the
 * context's own).  A march that has to build its scene's exact-skip bound
 * table builds it on a second stream of the context while it splats, and the
 * march's stream waits for it before the march kernels; fm_scene_destroy and
 * a grid rebuild that grows the scene's tables wait for both streams of the
 * context.  A scene is not updated or destroyed while a march on another
 * stream still reads it.
 */
#ifndef FLUIDMARCH_H
#define FLUIDMARCH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------
 * The reference has no status codes (SPDLOG_ERROR + continue, HZ_ASSERT);
 * every fm_* call returns one of these and keeps a message for
 * fm_last_error(). */
#define FM_OK 0
#define FM_ERR_INVALID 1  /* bad argument: null handle, N == 0, non-finite input, ... */
#define FM_ERR_CUDA 2     /* a CUDA call failed, or no CUDA device */
#define FM_ERR_TIMEOUT 3  /* fm_sync gave up waiting */
#define FM_ERR_OOM 4      /* device or pinned allocation failed */
#define FM_ERR_DEVICE 5   /* a kernel reported an error through its status word */

#define FM_MEM_HOST 0     /* pointer is host memory (pageable or pinned) */
#define FM_MEM_DEVICE 1   /* pointer is device memory of the context's device */

/* skip modes (march parameter) */
#define FM_SKIP_OFF 0        /* evaluate the density at every sample (reference parity gate) */
#define FM_SKIP_EXACT 1      /* skip samples whose bound box (an eighth of a cell per axis) has
                                a density upper bound below iso; same results as FM_SKIP_OFF.
                                The scene's bound table is built by its first such march
                                (boxes of a quarter cell, then those near the iso surface
                                refined into eighths) and serves marches at that iso or a
                                lower one; a march at a higher iso builds it again. */
#define FM_SKIP_REFERENCE 2  /* the reference's skip: flag = own-cell count * W0 > 1, jump to the
                                cell's exit plus one step (RayMarcher.cpp:281-306) */

/* march flags */
#define FM_MARCH_EXTERNAL_DEPTH 1 /* take ray-start depths from fm_frame_out.start_depth
                                     instead of splatting them (reference signature mode) */
#define FM_MARCH_PROPOSAL 2       /* march first inside the interval the context's learned
                                     proposal (fm_set_proposal) predicts; where it holds no
                                     crossing, march the rest of the ray (skip mode off or
                                     exact only) */

#define FM_MARCH_ANISOTROPIC 4    /* the reference's anisotropic march (RayMarcher.cpp:346-423):
                                     per-sample WPCA kernels with the context's
                                     fm_aniso_params (fm_set_anisotropy); no proposal.
                                     FM_SKIP_EXACT skips the samples whose bound box has
                                     no particle within the support radius (density
                                     exactly 0; iso > 0): same results as FM_SKIP_OFF */

/* learned proposal: features per ray and MLP parameter count */
#define FM_PROPOSAL_FEATURES 32
#define FM_PROPOSAL_PARAMS 6402

typedef struct fm_ctx fm_ctx;
typedef struct fm_scene fm_scene;

/* Camera: what RayMarcher::Prepare reads from CameraController3D
 * (RayMarcher.cpp:95-96: Position, InvProjectionView) plus what the depth
 * pass (DepthRenderPass.cpp:245-247: View, Projection) and the composition
 * pass (CompositionRenderPass.cpp:315-321: InvProjectionView, Position,
 * System[2]) read.  The image size replaces Vulkan.SwapchainExtent
 * (RayMarcher.cpp:86-89). */
typedef struct fm_camera {
    float view[16];
    float proj[16];
    float inv_proj_view[16];
    float position[3];
    int32_t width;
    int32_t height;
} fm_camera;

/* March settings: VisualizationSettings (RayMarcher.h:12-26) fields used by
 * the isotropic path, plus bisection and skip mode. */
typedef struct fm_march_params {
    float iso_density;    /* IsoDensity: hit when density >= iso_density */
    float step_size;      /* StepSize (world units) */
    int32_t max_steps;    /* MaxSteps */
    int32_t bisect_iters; /* 0 = reference behaviour (first sample with rho >= iso) */
    int32_t skip_mode;    /* FM_SKIP_* */
    int32_t flags;        /* FM_MARCH_* */
} fm_march_params;

/* Per-pixel outputs (any pointer may be NULL to skip that output).  The
 * reference writes glm::vec4 positions/normals (RayMarcher.cpp:330,338) into
 * caller-owned W*H buffers; colour is the composition pass
 * (composition.frag:132-184).  Pixel index = y * width + x, y = 0 at the top. */
typedef struct fm_frame_out {
    float* position;          /* 4 floats/pixel: (hit, 1) or 0 on miss */
    float* normal;            /* 4 floats/pixel: (n, 1) or 0 on miss */
    float* depth;             /* 1 float/pixel: |hit - camera| or 0 on miss */
    float* colour;            /* 4 floats/pixel: shaded RGBA */
    float* start_depth;       /* 1 float/pixel: splat depth written (or read with
                                 FM_MARCH_EXTERNAL_DEPTH); clear value 1.0 = no particle */
} fm_frame_out;

/* Grid of a scene: Frame::m_Min/m_Max (Dataset.cpp:78-92) and
 * DensityGrid (Dataset.cpp:94-104). */
typedef struct fm_grid_info {
    float min[3];
    float max[3];
    float cell_width;
    float inv_cell_width;
    int32_t dims[3];
    int32_t pad;
    uint64_t n_particles;
    uint64_t n_cells;
} fm_grid_info;

/* Counters a march can accumulate (fm_march_stats). */
typedef struct fm_march_stats {
    uint64_t rays;          /* pixels marched */
    uint64_t started;       /* rays whose start depth != 1.0 */
    uint64_t hits;
    uint64_t evals;         /* density evaluations (march samples + bisection + normal) */
    uint64_t candidates;    /* particles in the 27 cells of every evaluation */
    uint64_t skipped;       /* samples skipped by FM_SKIP_EXACT */
    uint64_t tested;        /* particles actually tested: those of sub-cells within reach */
    uint64_t streamed;      /* particles a warp streamed for its lanes (shared candidate stream) */
    uint64_t deferred;      /* rays finished by the long-ray pass */
    uint64_t proposed;      /* rays that started inside a proposed interval (FM_MARCH_PROPOSAL) */
    uint64_t fallbacks;     /* of those, rays that went back for the samples before the interval */
    uint64_t regrouped;     /* rays the first pass handed to the regrouped second pass */
} fm_march_stats;

/* ---- context ------------------------------------------------------------ */

/* RayMarcher::RayMarcher (RayMarcher.cpp:66-69): create a context bound to a
 * CUDA device, with its own non-blocking stream. */
int fm_create(fm_ctx** out, int device);
/* RayMarcher::Exit (RayMarcher.cpp:71-74): wait for work, free everything,
 * including the scenes of this context that were not destroyed yet (their
 * handles become invalid; destroy scenes first to keep them usable). */
void fm_destroy(fm_ctx* ctx);
/* Message of the last failing call on this context (never NULL). */
const char* fm_last_error(const fm_ctx* ctx);
/* The same message under the name a binding of the reference's renderer may expect. */
const char* fm_last_error_string(const fm_ctx* ctx);
/* The context's stream as a cudaStream_t. */
void* fm_stream(fm_ctx* ctx);
/* Wait for all work on the context's stream; FM_ERR_TIMEOUT after timeout_ms
 * (< 0: wait forever).  Also reports kernel status words (FM_ERR_DEVICE). */
int fm_sync(fm_ctx* ctx, int timeout_ms);
/* RayMarcher::IsDone (RayMarcher.h:44, ThreadPool.cpp:33-36): 1 when the
 * stream is idle, 0 when work is pending, < 0 on error.  Unlike the reference,
 * "done" means every output has been written. */
int fm_query(fm_ctx* ctx);
/* Pinned (page-locked, mapped) host memory.  March outputs that lie inside
 * such a block are written by the kernels directly, with no copy after the
 * march; when every host buffer of an fm_march call (outputs and start depth)
 * lies in such blocks the call is asynchronous, as with device buffers: poll
 * fm_query, finish with fm_sync (which also reports kernel status).
 * fm_host_free waits for the device before it frees the block. */
int fm_host_alloc(fm_ctx* ctx, size_t bytes, void** out);
void fm_host_free(fm_ctx* ctx, void* p);

/* ---- scenes ------------------------------------------------------------- */

/* Frame::Frame (Dataset.cpp:9-24): upload n particles (xyz at a stride of
 * `stride` floats, >= 3) and build the uniform grid with cell width
 * support_radius (Dataset::ParticleRadius): AABB, per-particle cell
 * index (bit-identical to QueryDensityGrid), stable counting sort by cell,
 * cell start table.  Synchronous.  Non-finite positions are rejected. */
int fm_scene_create(fm_ctx* ctx, const float* xyz, uint64_t n, uint32_t stride, float support_radius,
                    int mem, fm_scene** out);
/* Rebuild an existing scene from new positions (same n or fewer, same
 * radius): a new frame of the same dataset (Dataset::ReadFile adds one,
 * Dataset.cpp:292-306). */
int fm_scene_update(fm_scene* scene, const float* xyz, uint64_t n, uint32_t stride, int mem);
/* fm_scene_create from host memory (the reference builds a Frame from a host
 * std::vector of positions, Dataset.cpp:9-24). */
int fm_scene_upload(fm_ctx* ctx, const float* xyz, uint64_t n, int32_t stride_floats, float support_radius,
                    fm_scene** out);
void fm_scene_destroy(fm_scene* scene);
int fm_scene_grid(const fm_scene* scene, fm_grid_info* out);
/* Download the grid build (host pointers; any may be NULL):
 *   cell[n]         linear cell of each input particle (QueryDensityGrid index)
 *   sorted_index[n] input index of each cell-sorted particle
 *   cell_start[n_cells + 1]
 *   sorted_xyzw[4n] cell-sorted positions (w = 0) */
int fm_scene_download(const fm_scene* scene, uint32_t* cell, uint32_t* sorted_index, uint32_t* cell_start,
                      float* sorted_xyzw);

/* Grid build that allocates nothing.  No counterpart in the reference: it is
 * for callers that cannot or must not allocate device memory (a renderer that
 * reserves all its memory up front, a plugin inside a host application's
 * memory budget).  Same results as the grid build of fm_scene_create, on the
 * current CUDA device and context, on `stream`:
 *   xyz            device, n particles at a stride of `stride` floats (>= 3)
 *   sorted_xyzw    device, 4n floats, 16-byte aligned: sorted positions (w = 0);
 *                  also holds the sort's temporaries until the last step
 *   cell           device, n: cell of each input particle (QueryDensityGrid index)
 *   sorted_index   device, n: input index of each sorted particle
 *   sub_start      device, sub_start_capacity entries: the 8 * n_cells + 1
 *                  sub-cell starts (cell c = [sub_start[8c], sub_start[8c+8]))
 *   info           host: grid origin, dims, n_cells (also filled when the
 *                  capacity is too small, so a caller can size sub_start)
 * The five device buffers must be memory of the current device or managed
 * memory (FM_ERR_INVALID otherwise); their sizes are the caller's promise.
 * Limits: n <= 2^21 particles, n_cells <= 2^21; FM_ERR_INVALID beyond them.
 * Scratch lives in one device array of about 1.1 MB inside the library (held
 * by every device that loads it until the process exits), shared by all
 * calls: calls that overlap on the GPU race and must be serialised.  The
 * first call in a CUDA context looks up that array's address in the context
 * (a driver-API context of the host application works as well as the
 * device's primary context).  Each call synchronises `stream` once (to read
 * the bounding box); the rest is enqueued asynchronously.  Returns FM_OK,
 * FM_ERR_INVALID or FM_ERR_CUDA; there is no context and no message. */
int fm_grid_build_noalloc(const float* xyz, uint64_t n, uint32_t stride, float support_radius, float* sorted_xyzw,
                          uint32_t* cell, uint32_t* sorted_index, uint32_t* sub_start, uint64_t sub_start_capacity,
                          fm_grid_info* info, void* stream);

/* ---- rendering ---------------------------------------------------------- */

/* Depth pass (DepthRenderPass, depth.vert/depth.frag): splat every particle
 * as a camera-facing sphere of radius support_radius into a W*H depth buffer
 * cleared to 1.0 (LESS test).  Asynchronous on `stream` (NULL = context
 * stream). */
int fm_splat_depth(fm_ctx* ctx, const fm_scene* scene, const fm_camera* cam, float* depth, int mem, void* stream);

/* RayMarcher::Start + PerPixel_Isotropic (RayMarcher.cpp:102-112,256-344)
 * plus the composition shading: splat (unless FM_MARCH_EXTERNAL_DEPTH),
 * march every pixel, bisect, take the gradient normal, shade.  Asynchronous
 * for device outputs and for host buffers that all lie in fm_host_alloc
 * blocks; for other host buffers the call returns once they are written. */
int fm_march(fm_ctx* ctx, const fm_scene* scene, const fm_camera* cam, const fm_march_params* params,
             const fm_frame_out* out, int mem, void* stream);

/* Anisotropic kernels: VisualizationSettings k_n, k_r, k_s, N_eps
 * (RayMarcher.h:12-26; defaults AdvancedRenderer.cpp:23-27) and the
 * Dataset's particleRadiusMultiplier (extended radius = radius_mult x support
 * radius, Dataset.cpp:175; main.cpp default 2). */
typedef struct fm_aniso_params {
    float radius_mult;
    float k_n;
    float k_r;
    float k_s;
    int32_t n_eps;
    int32_t reserved; /* 0 */
} fm_aniso_params;
/* The parameters FM_MARCH_ANISOTROPIC uses on this context (NULL: 2, 0.5, 2, 2000, 1). */
int fm_set_anisotropy(fm_ctx* ctx, const fm_aniso_params* params);

/* DiskRenderer::ComputeDensity (DiskRenderer.cpp:180-193): SPH density at n
 * points (xyz at a stride of `stride` floats, >= 3) into out[n], summed over
 * the 27 grid cells around each point in the march's order (bit-identical to
 * the march's density at the same point).  Host buffers: synchronous; device
 * buffers: asynchronous on `stream`. */
int fm_density(fm_ctx* ctx, const fm_scene* scene, const float* xyz, uint64_t n, uint32_t stride, float* out, int mem,
               void* stream);

/* Counters of the last fm_march / fm_batch_run on this context (enable with
 * fm_set_stats(ctx, 1); counting costs time, keep it off when timing). */
int fm_set_stats(fm_ctx* ctx, int enable);
int fm_march_stats_get(fm_ctx* ctx, fm_march_stats* out);

/* ---- work split and batches --------------------------------------------
 * No counterpart in the reference, which renders one view per Start() with a
 * thread pool over pixels (RayMarcher.cpp:102-112, ThreadPool.cpp:5-55).  */

/* How the march splits an image among warps.  Results do not depend on it. */
typedef struct fm_tile_config {
    int32_t tile_width;      /* pixels per tile row: 1, 2, 4, 8, 16 or 32; a tile
                                is tile_width x (32 / tile_width) pixels */
    int32_t tiles_per_claim; /* tiles a warp takes at a time: 1..16 */
    int32_t defer_iters;     /* density sums a warp runs for one tile before the
                                rays it still has go to the long-ray pass: 1..4096;
                                0 = 12 for fm_march with the exact skip, else 15
                                (batches: 24) */
    int32_t long_queue;      /* entries of the long-ray queue; 0 = pixels / 4 + 65536.
                                Rays that find it full stay with their warp. */
    int32_t defer_lanes;     /* a warp also defers its rays once at most this many are
                                still active: 0..31 */
    int32_t regroup_iters;   /* deferred rays are sorted by tile and marched again 32 to
                                a warp for this many sums before the warp-per-ray pass
                                takes the rest: 0 (no second pass)..4096 */
} fm_tile_config;

/* Work split of fm_march on this context (default 8, 1, 0, 0, 2, 0). */
int fm_set_tile_config(fm_ctx* ctx, const fm_tile_config* cfg);
int fm_get_tile_config(const fm_ctx* ctx, fm_tile_config* out);

/* One view of a batch: a scene seen from a camera with its own march
 * settings.  Output pointers are DEVICE memory (NULL skips an output);
 * start_depth may be NULL (the batch keeps the splat depths itself).  Every
 * view is splatted: params.flags may hold FM_MARCH_PROPOSAL (the batch copies
 * the context's proposal at creation) or FM_MARCH_ANISOTROPIC (the batch
 * copies the context's fm_set_anisotropy settings), not
 * FM_MARCH_EXTERNAL_DEPTH. */
typedef struct fm_view {
    const fm_scene* scene;
    fm_camera camera;
    fm_march_params params;
    fm_frame_out out;
} fm_view;

typedef struct fm_batch fm_batch;

typedef struct fm_batch_info {
    int32_t n_views;
    int32_t graph_nodes;     /* kernel and memset nodes of the captured graph */
    uint64_t pixels;         /* sum of W * H over the views */
    uint64_t particles;      /* sum of the views' particle counts */
    uint64_t tiles;          /* march tiles of the whole batch */
    fm_tile_config config;   /* work split in use */
} fm_batch_info;

/* Prepare a batch of views: all views are splatted and marched by one launch
 * per pass (fill, sampled splat, tile maxima, cull, survivor splat, proposal
 * when a view has one, march, long rays, anisotropic march when a view is
 * anisotropic), captured once into a CUDA graph.  The views' scenes and output
 * buffers are bound at creation: after fm_scene_update of one of its scenes,
 * call fm_batch_refresh.  cfg NULL: the context's work split.  Synchronous. */
int fm_batch_create(fm_ctx* ctx, const fm_view* views, int32_t n_views, const fm_tile_config* cfg, fm_batch** out);
/* Render every view: one graph launch on `stream` (NULL = context stream),
 * asynchronous.  With counters enabled (fm_set_stats) the passes are launched
 * without the graph and counted. */
int fm_batch_run(fm_batch* batch, void* stream);
/* Re-read the scenes' grids and re-capture the graph (synchronous). */
int fm_batch_refresh(fm_batch* batch);
/* Time the batch under candidate work splits (`reps` timed runs each after
 * one warm-up; cands NULL: a built-in set of tile shapes, claims and defer
 * limits), keep the fastest, re-capture.  best / best_ms may be NULL.
 * Synchronous; the outputs hold the last run's results (identical for every
 * split). */
int fm_batch_autotune(fm_batch* batch, const fm_tile_config* cands, int32_t n_cands, int32_t reps,
                      fm_tile_config* best, float* best_ms);
int fm_batch_info_get(const fm_batch* batch, fm_batch_info* out);
void fm_batch_destroy(fm_batch* batch);
/* One-shot: create a batch, run it on `stream`, wait, destroy it. */
int fm_march_batch(fm_ctx* ctx, const fm_view* views, int32_t n_views, void* stream);

/* ---- learned hit-interval proposal -------------------------------------
 * No counterpart in the reference.  A 3-layer MLP (width 64, GELU) maps the
 * FM_PROPOSAL_FEATURES features of a ray (16 samples of a 64^3 occupancy grid
 * along the ray, the 1/8-resolution splat depth, the direction, the start
 * point in the scene box) to an interval (near, far), in support radii past
 * the ray start.  With FM_MARCH_PROPOSAL the march evaluates only the samples
 * of its own sample lattice inside [near - margin_lo, far + margin_hi] and
 * restarts as the full march when that interval holds no crossing or its first
 * sample is already inside: hit masks equal the full march's, a depth differs
 * only where the fluid is crossed before near.  Inference runs on the BF16
 * tensor cores with FP32 accumulation.
 *
 * Parameters: FM_PROPOSAL_PARAMS floats, W1[64][32], b1[64], W2[64][64],
 * b2[64], W3[2][64], b3[2] (W[out][in]). */
typedef struct fm_proposal fm_proposal;
/* margin_lo / margin_hi widen every interval (support radii); rays whose
 * widened near is below min_near (support radii) run the full march. */
int fm_proposal_create(fm_ctx* ctx, const float* params, float margin_lo, float margin_hi, float min_near,
                       fm_proposal** out);
void fm_proposal_destroy(fm_proposal* p);
/* The proposal FM_MARCH_PROPOSAL uses on this context (NULL clears). */
int fm_set_proposal(fm_ctx* ctx, fm_proposal* p);
/* Features of every pixel's ray (training data), device buffers:
 *   start_depth  W*H splat depths (as fm_march writes them)
 *   features     W*H*FM_PROPOSAL_FEATURES floats (0 for pixels without a ray)
 *   t0           W*H ray-start distances from the camera (may be NULL) */
int fm_proposal_features(fm_ctx* ctx, const fm_scene* scene, const fm_camera* cam, const float* start_depth,
                         float* features, float* t0, void* stream);
/* Intervals the march would use, device buffers: intervals = W*H pairs
 * (first sample - 1, last sample) of the march's sample index, (0, -1) for a
 * full march; near_far = W*H raw (near, far) outputs (may be NULL).  The
 * usable intervals of every 8x4 pixel block start at the block's earliest
 * start, so that the rays of a march tile step together. */
int fm_proposal_intervals(fm_ctx* ctx, const fm_scene* scene, const fm_camera* cam, const fm_march_params* params,
                          const float* start_depth, int32_t* intervals, float* near_far, void* stream);

/* Judge: compare a march's per-pixel hit distances (fm_frame_out.depth, 0 =
 * miss) with a reference march's, device buffers, synchronous. */
typedef struct fm_judge_result {
    uint64_t pixels;
    uint64_t hits_ref;
    uint64_t hits_test;
    uint64_t mask_mismatch;  /* pixels hit in one and missed in the other */
    uint64_t within_tol;     /* pixels hit in both with |depth difference| <= tol */
    float max_err;           /* largest |depth difference| over pixels hit in both */
    float tol;
} fm_judge_result;
int fm_judge(fm_ctx* ctx, const float* depth_ref, const float* depth_test, uint64_t n, float tol,
             fm_judge_result* out, void* stream);

/* Per-frame judge of the learned march.  No counterpart in the reference (the
 * learned proposal is an addition).  With stride > 0, every FM_MARCH_PROPOSAL
 * march of this context also marches the started rays of a pixel sample
 * (about 1 in `stride` 8x4 pixel blocks, drawn by a hash of the block index
 * and a frame counter, so every frame judges other pixels) with the plain march -- same
 * iso, step, steps, bisection and skip mode -- right after the learned march on
 * the same stream, and compares their hit distances with the learned march's
 * on the device: hit-mask mismatches, hits within `tol` (world units) and the
 * largest difference accumulate until fm_judge_frames reads them.  The cost is
 * part of the learned march.  stride 0 turns the judge off. */
int fm_set_judge(fm_ctx* ctx, uint32_t stride, float tol);
typedef struct fm_frame_judge {
    uint64_t frames;         /* learned marches judged since the last reset */
    uint64_t sampled;        /* started rays in the samples */
    uint64_t hits_ref;       /* of those, hits of the plain march */
    uint64_t hits_test;      /* hits of the learned march */
    uint64_t mask_mismatch;  /* hit in one march and missed in the other */
    uint64_t within_tol;     /* hit in both with |depth difference| <= tol */
    float max_err;           /* largest |depth difference| over rays hit in both */
    float tol;
} fm_frame_judge;
/* What the per-frame judge accumulated (waits for the context's work);
 * reset != 0 clears it afterwards. */
int fm_judge_frames(fm_ctx* ctx, fm_frame_judge* out, int reset);

/* Training of the proposal: FP32 forward, backward and Adam kernels.  Loss:
 * pinball (quantile) loss of near at quantile tau_lo and of far at tau_hi
 * against the first-hit distance (support radii past the ray start). */
typedef struct fm_trainer fm_trainer;
/* init NULL: seeded uniform initialisation (biases 0). */
int fm_trainer_create(fm_ctx* ctx, uint64_t seed, const float* init, fm_trainer** out);
void fm_trainer_destroy(fm_trainer* t);
/* One Adam step on a batch of n rays (device buffers: n*FM_PROPOSAL_FEATURES
 * features, n targets); loss (host, may be NULL) = mean loss before the step. */
int fm_trainer_step(fm_trainer* t, const float* features, const float* targets, uint32_t n, float lr, float tau_lo,
                    float tau_hi, float* loss);
/* FP32 outputs (near, far) of the current parameters: out = n*2 floats (device). */
int fm_trainer_predict(fm_trainer* t, const float* features, uint32_t n, float* out);
int fm_trainer_params(fm_trainer* t, float* host_params);
/* Checkpoint: state = 3 * FM_PROPOSAL_PARAMS floats (parameters | Adam first
 * moments | second moments) and the Adam step count.  Gradients are reduced in
 * a fixed order, so a trainer restored with fm_trainer_set_state continues
 * bit for bit as the one that wrote the state. */
int fm_trainer_get_state(fm_trainer* t, float* host_state, int64_t* step);
int fm_trainer_set_state(fm_trainer* t, const float* host_state, int64_t step);

/* ---- Particle files (Dataset.cpp:169-227, Dataset::ReadFile :292-306) ----
 * Houdini classic BGEO, version 5, plain or gzip-compressed (detected by the
 * gzip magic), the format the reference reads through Partio
 * (vendor/partio/src/io/BGEO.cpp readBGEO): the position of every point (the
 * first three words of its big-endian record).  Other point attributes are
 * skipped, as Dataset::ReadFile ignores them. */
typedef struct fm_bgeo_info {
    uint64_t points;
    uint32_t record_words;  /* 32-bit words per point record: 4 (x y z w) + attribute sizes */
    uint32_t attributes;    /* point attributes besides position */
    uint64_t file_bytes;
    uint64_t data_bytes;    /* after decompression (0 when only the header was read) */
    int32_t compressed;     /* 1: gzip */
    int32_t reserved;
} fm_bgeo_info;

/* Host read, no GPU needed: the positions of the first min(capacity, points)
 * points into xyz (3 floats each; xyz NULL: header only).  err (may be NULL):
 * the message of a failure.  A header read rejects a point count the file
 * cannot hold for plain files and for gzip files below ~4 MB (whose size
 * field is exact); a larger gzip file's count is checked when it is decoded. */
int fm_bgeo_read(const char* path, float* xyz, uint64_t capacity, fm_bgeo_info* info, char* err, uint64_t err_len);
/* First member of a gzip stream (RFC 1952), CRC-32 and length checked.
 * out_len = the decoded size; FM_ERR_INVALID when it exceeds out_cap (nothing
 * copied) or the stream is corrupt.  No GPU needed. */
int fm_gunzip(const void* in, uint64_t in_len, void* out, uint64_t out_cap, uint64_t* out_len);
/* A scene from a BGEO file: decompressed on the host, the point records
 * copied to the device, positions byte-swapped by a kernel, then the grid
 * build of fm_scene_create (replaces Partio::read + Frame::Frame).  Synchronous. */
int fm_scene_create_bgeo(fm_ctx* ctx, const char* path, float support_radius, fm_scene** out);

/* A numbered series prefix + i + suffix, i = 1, 2, ... until a file is
 * missing or i > count (count < 0: no limit), as the Dataset constructor
 * collects it.  threads > 0 host threads decode the 2 * threads frames after
 * the one last asked for (autoplay, AdvancedRenderer.cpp:281-297). */
typedef struct fm_dataset fm_dataset;
int fm_dataset_open(const char* prefix, const char* suffix, int32_t count, int32_t threads, fm_dataset** out,
                    char* err, uint64_t err_len);
int32_t fm_dataset_frames(const fm_dataset* ds);
const char* fm_dataset_path(const fm_dataset* ds, int32_t i);
/* Header of frame i (data_bytes 0). */
int fm_dataset_frame_info(fm_dataset* ds, int32_t i, fm_bgeo_info* info);
/* Largest particle count over the frames (Dataset::MaxParticles, Dataset.cpp:222-224). */
int fm_dataset_max_particles(fm_dataset* ds, uint64_t* out);
/* Positions of frame i on the host (n = its particle count). */
int fm_dataset_read(fm_dataset* ds, int32_t i, float* xyz, uint64_t capacity, uint64_t* n);
/* Frame i as a scene.  *scene NULL: created.  Otherwise rebuilt in place
 * (fm_scene_update) when frame i has at most the particles it was created
 * with and the same support radius, else replaced (the handle changes;
 * batches holding the old one must be recreated).  Synchronous.  Errors go
 * to fm_last_error(ctx). */
int fm_dataset_scene(fm_dataset* ds, fm_ctx* ctx, int32_t i, float support_radius, fm_scene** scene);
const char* fm_dataset_last_error(const fm_dataset* ds);
void fm_dataset_close(fm_dataset* ds);

/* The depth Gaussian blur pass (GaussRenderPass.cpp:13-57,347-355, gauss.frag):
 * out = sum over i, j = -n..n of ComputeGaussKernel's weight(|i|, |j|) times the
 * depth image sampled at the pixel centre's UV + (i, j) * (spread / width,
 * spread / height), linear filtering with clamp-to-edge (8 sub-texel bits).
 * n in [0, 31] (the reference's GaussN, default 8), spread > 0 (the "Blur
 * spread" slider, default 1: every tap reads one texel).  Host buffers are
 * staged and the call returns when out is written; device buffers run on
 * `stream`. */
int fm_depth_blur(fm_ctx* ctx, const float* depth, float* out, int32_t width, int32_t height, int32_t n,
                  float spread, int mem, void* stream);

/* Diagnostics for failure detection: runs the bounded mbarrier wait of the
 * tensor-core kernels on a barrier that never completes.  The wait gives up
 * after `polls` polls (1 .. 2^22), the kernel sets status bit 8 as the
 * proposal kernel does on a timeout, and the call returns FM_ERR_DEVICE with
 * the status word in fm_last_error; the context stays usable. */
int fm_selftest_wait_timeout(fm_ctx* ctx, uint32_t polls);

/* Library version (major * 10000 + minor * 100 + patch). */
int fm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FLUIDMARCH_H */
