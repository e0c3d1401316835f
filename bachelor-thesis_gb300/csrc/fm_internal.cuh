// fm_internal.cuh -- shared device structures and exact FP32 helpers.
//
// Every translation unit of libfluidmarch is compiled with --fmad=false, so a
// plain expression `a * b + c` is two separately rounded operations, exactly
// as the reference's /fp:precise build and glm 0.9.9 evaluate it.  That makes
// the cell index, the march samples, the kernel sums and the shading
// bit-identical to the reference formulas for the same summation order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/fluidmarch.h"

namespace fm {

constexpr int kWarp = 32;
constexpr int kBoundDiv = 8;            // exact-skip bound boxes per cell and axis
constexpr int kBoundBoxes = kBoundDiv * kBoundDiv * kBoundDiv;
constexpr int kProposalOcc = 64;        // occupancy grid resolution of the proposal
constexpr int kProposalFeatures = FM_PROPOSAL_FEATURES;
constexpr int kProposalParams = FM_PROPOSAL_PARAMS;
constexpr unsigned kWorkSlots = 64;
constexpr int kStatSlots = 16;

// Uniform grid of a scene (Frame::m_Min, DensityGrid; Dataset.cpp:78-104).
struct GridDev {
    float min[3];
    float inv;   // 1.0f / cell
    float cell;  // cell width = support radius
    int dims[3];
    uint32_t nsub;                        // 8 * n_cells + 1 (entries of sub)
    const float4* __restrict__ pts;       // sorted particles (w = 0): cell, 2x2x2 sub-cell, input index
    const uint32_t* __restrict__ sub;     // 8 * n_cells + 1 sub-cell starts; cell c = [sub[8c], sub[8c+8])
    const float* __restrict__ bound;      // per bound box density upper bound (FM_SKIP_EXACT) or null
    const uint8_t* __restrict__ flag;     // per-cell reference skip flag (FM_SKIP_REFERENCE) or null
    float zlo[3], zhi[3];                 // zero-density box: outside it no particle is within the support radius
};

// Cubic spline constants, Kernel.cpp:8-14 (h = support radius).
struct KernelDev {
    float h, h2, hinv, sig;
};

// Host: constants evaluated in FP32 in the reference's order.
inline KernelDev make_kernel(float h) {
    KernelDev k;
    k.h = h;
    k.h2 = h * h;
    k.hinv = 1.0f / h;
    const float pi = 3.14159265358979323846f;
    k.sig = 8.0f / (((pi * h) * h) * h);
    return k;
}

// glm dot for vec3: (x*x' + y*y') + z*z'
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return (ax * bx + ay * by) + az * bz;
}

// CubicSplineKernel::W for q2 = dot(r, r) < h2 (Kernel.cpp:16-32).
__device__ __forceinline__ float w_in(const KernelDev& k, float q2) {
    float q = sqrtf(q2) * k.hinv;
    // both branches of the reference's kernel, then a select: lanes of a warp
    // fall on either side of q = 0.5, and a select costs less than two paths
    float q_ = 1.0f - q;
    float a = k.sig * (((2.0f * q_) * q_) * q_);
    float b = k.sig * (6.0f * (((q * q) * q) - (q * q)) + 1.0f);
    return q >= 0.5f ? a : b;
}

// CubicSplineKernel::gradW for 0 < rn < h2 (Kernel.cpp:34-52): the term itself.
__device__ __forceinline__ void gradw_term(const KernelDev& k, float rx, float ry, float rz, float rn, float& tx,
                                           float& ty, float& tz) {
    float rl = sqrtf(rn);
    float q = rl * k.hinv;
    float inv = 1.0f / sqrtf(rn);  // normalize(r) = r * inversesqrt(dot(r, r))
    float den = rl * k.h;
    float nx = (rx * inv) / den, ny = (ry * inv) / den, nz = (rz * inv) / den;
    float ax, ay, az, s;
    if (q >= 0.5f) {
        float q_ = 1.0f - q;
        s = (6.0f * q_) * q_;
        float ns = -k.sig;
        ax = ns * nx; ay = ns * ny; az = ns * nz;
    } else {
        s = 6.0f * (((3.0f * q) * q) - (2.0f * q));
        ax = k.sig * nx; ay = k.sig * ny; az = k.sig * nz;
    }
    tx = ax * s;
    ty = ay * s;
    tz = az * s;
}

// CubicSplineKernel::gradW for 0 < rn < h2 (Kernel.cpp:34-52), accumulated
// into g with glm's component order.
__device__ __forceinline__ void gradw_acc(const KernelDev& k, float rx, float ry, float rz, float rn, float& gx,
                                          float& gy, float& gz) {
    float rl = sqrtf(rn);
    float q = rl * k.hinv;
    float inv = 1.0f / sqrtf(rn);  // normalize(r) = r * inversesqrt(dot(r, r))
    float den = rl * k.h;
    float nx = (rx * inv) / den, ny = (ry * inv) / den, nz = (rz * inv) / den;
    float ax, ay, az, s;
    if (q >= 0.5f) {
        float q_ = 1.0f - q;
        s = (6.0f * q_) * q_;
        float ns = -k.sig;
        ax = ns * nx; ay = ns * ny; az = ns * nz;
    } else {
        s = 6.0f * (((3.0f * q) * q) - (2.0f * q));
        ax = k.sig * nx; ay = k.sig * ny; az = k.sig * nz;
    }
    gx = gx + ax * s;
    gy = gy + ay * s;
    gz = gz + az * s;
}

// Sample -> cell (QueryDensityGrid formula, Dataset.cpp:28-33).  false when
// the sample is so far outside that its 27 neighbourhood misses the grid, or
// non-finite.
__device__ __forceinline__ bool sample_cell(const GridDev& g, float px, float py, float pz, int& cx, int& cy,
                                            int& cz) {
    float fx = floorf((px - g.min[0]) * g.inv);
    float fy = floorf((py - g.min[1]) * g.inv);
    float fz = floorf((pz - g.min[2]) * g.inv);
    if (!(fx >= -2.0f && fx <= (float)g.dims[0] + 1.0f)) return false;
    if (!(fy >= -2.0f && fy <= (float)g.dims[1] + 1.0f)) return false;
    if (!(fz >= -2.0f && fz <= (float)g.dims[2] + 1.0f)) return false;
    cx = (int)fx;
    cy = (int)fy;
    cz = (int)fz;
    return true;
}

// True when sample p lies beyond the grid's evaluation range (the range in
// which sample_cell succeeds) on some axis and the step s points further away
// on that axis.  FP32 addition of a same-signed step is monotone, so every
// later sample stays out there and has density exactly 0: the march can stop
// with a miss and produce the same outputs as running to max_steps.
__device__ __forceinline__ bool outside_forever(const GridDev& g, float px, float py, float pz, float sx, float sy,
                                                float sz) {
    const float p[3] = {px, py, pz}, s[3] = {sx, sy, sz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = floorf((p[a] - g.min[a]) * g.inv);
        if (f > (float)g.dims[a] + 1.0f && s[a] >= 0.0f) return true;
        if (f < -2.0f && s[a] <= 0.0f) return true;
    }
    return false;
}

// The grid spans the particles' bounding box padded by the support radius H
// (Dataset.cpp:89-92), so a sample farther than H beyond that box on some axis
// has no particle within H: its FP32 density is exactly 0 (every term's
// squared distance rounds to at least H^2).  zlo / zhi are the padded box grown
// by a slack of 1e-4 H + 1e-6 max|coordinate|, which covers the rounding of the
// padding, of the differences and of the squared distances.
__device__ __forceinline__ bool zero_density(const GridDev& g, float px, float py, float pz) {
    return px < g.zlo[0] || px > g.zhi[0] || py < g.zlo[1] || py > g.zhi[1] || pz < g.zlo[2] || pz > g.zhi[2];
}

// True when p is outside the zero-density box on an axis and the step moves
// further out on it: every later sample has density exactly 0.
__device__ __forceinline__ bool leaving_zero_box(const GridDev& g, float px, float py, float pz, float sx, float sy,
                                                 float sz) {
    return (px > g.zhi[0] && sx >= 0.0f) || (px < g.zlo[0] && sx <= 0.0f) || (py > g.zhi[1] && sy >= 0.0f) ||
           (py < g.zlo[1] && sy <= 0.0f) || (pz > g.zhi[2] && sz >= 0.0f) || (pz < g.zlo[2] && sz <= 0.0f);
}

// ---- host-side objects ------------------------------------------------------

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

// Work split of the march: tile shape, tiles per claim, iterations before
// the rays a warp has left are deferred to the long-ray pass.
struct TileConfig {
    int tw_log2 = 3;  // 8x4 pixels
    int claim = 1;
    int cap = 0;          // shared-stream sums before deferral; 0: 12 (single view, exact skip), 15, 24 (batches)
    int lanes = 2;        // a warp defers its rays once at most this many are active
    int cap2 = 0;         // iterations of the regrouped second pass (0: no second pass)
    uint32_t qlimit = 0;  // long-ray queue entries (0: long_queue_entries of the pixels)
};

}  // namespace fm

struct fm_batch;

struct fm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // a march that builds the scene's bound table does so on `side`, next to
    // its splat; the march waits for it through ev_join
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;
    int sm_count = 0;
    // staging buffers for host in/outputs (grown on demand)
    fm::DevBuf stage[6];
    // device status word + stats accumulators
    unsigned int* d_status = nullptr;
    unsigned long long* d_stats = nullptr;  // kStatSlots counters
    // work counters of persistent kernels: kWorkSlots slots of 32 words (one
    // 128-byte line each), a fresh slot per launch
    unsigned int* d_work = nullptr;
    unsigned int work_slot = 0;
    int stats_enabled = 0;
    fm_march_stats last_stats{};
    // scratch for grid builds
    fm::DevBuf scratch[8];
    // the key counts and the bounds accumulator of a grid build return to their
    // initial state at the end of every build; they are set again when they
    // were reallocated or a build stopped in between
    bool grid_scratch_dirty = true;
    // long-ray queue of the march (64 B per entry, long_queue_entries(pixels)
    // entries for the largest view so far)
    fm::DevBuf longq;
    fm::DevBuf aniso_list;  // started pixels of an anisotropic march (one ray per claim)
    // regrouped second pass: second queue, sort counters, scan temporaries, order
    fm::DevBuf longq2, rg_keys, rg_tmp, rg_order;
    // splat depth tile maxima (4 B per 8x8 tile) and the list of particles that
    // survive the tile test; renders of one context on different streams must
    // not overlap
    fm::DevBuf hiz;
    fm::DevBuf splat_list;
    // learned proposal: the one fm_march uses with FM_MARCH_PROPOSAL, per-pixel
    // intervals, occupancy counts, low-resolution depth, judge counters
    fm_proposal* proposal = nullptr;
    fm::DevBuf prop_ivl, prop_scratch, prop_low, prop_judge;
    // per-frame judge of learned marches (fm_set_judge): sample stride, depth
    // tolerance, frames judged so far (seeds the sample), sample start plane,
    // plain-march and learned-march hit distances, counters
    uint32_t judge_stride = 0;
    float judge_tol = 0.0f;
    uint64_t judge_seq = 0;
    fm::DevBuf judge_z, judge_ref, judge_test, judge_acc;
    fm::DevBuf judge_longq;  // the sample march's long-ray queue (it runs next to the learned march)
    cudaEvent_t ev_jfork = nullptr, ev_jjoin = nullptr;
    fm::DevBuf file_rec, file_xyz;  // particle-file loader: point records, gathered positions
    fm::DevBuf blur_in, blur_out;   // depth blur staging for host buffers
    // live scenes of this context; fm_destroy frees the ones still alive
    std::vector<fm_scene*> scenes;
    // live batches of this context; fm_destroy frees the ones still alive
    std::vector<fm_batch*> batches;
    // work split of single-view marches (fm_set_tile_config)
    fm::TileConfig tile;
    // anisotropic kernels (fm_set_anisotropy)
    fm_aniso_params aniso{2.0f, 0.5f, 2.0f, 2000.0f, 1, 0};
    // source of scene generations (every successful build gets a new one)
    uint64_t gen_counter = 0;
    void* h_pinned_small = nullptr;  // 256 bytes of pinned memory for small readbacks
    // fm_host_alloc blocks: host address -> (bytes, device address of the mapping);
    // march outputs that lie inside one are written by the kernels directly
    std::map<uintptr_t, std::pair<size_t, void*>> host_allocs;
};

struct fm_scene {
    fm_ctx* ctx = nullptr;
    uint64_t n = 0;
    uint64_t capacity = 0;
    float support = 0.0f;
    float min[3], max[3];
    float inv = 0.0f;
    int dims[3] = {0, 0, 0};
    uint64_t ncells = 0;
    uint64_t cell_capacity = 0;
    float4* d_pts = nullptr;       // sorted by cell, sub-cell, input index
    uint32_t* d_cell = nullptr;    // cell of each input particle
    uint32_t* d_perm = nullptr;    // input index of each sorted particle
    uint32_t* d_sub = nullptr;     // 8 * ncells + 1 sub-cell starts
    float* d_bound = nullptr;      // exact-skip bound table, 8x8x8 boxes per cell (lazy)
    fm::DevBuf coarse;             // its 4x4x4 first level (64 bounds per cell)
    bool bound_fine = false;       // the shell boxes are refined (ensure_bound refines right after the first level)
    uint8_t* d_flag = nullptr;     // per-cell reference flag (lazy)
    bool bound_valid = false;      // built by the first exact-skip march after a build
    float bound_iso = 0.0f;        // the bound table holds +inf for boxes whose sum reached it
    bool flag_valid = false;
    uint64_t gen = 0;              // build generation: batches bound to an older one refuse to run
    uint16_t* d_occ = nullptr;     // 64^3 FP16 occupancy of the proposal (lazy)
    bool occ_valid = false;
};

namespace fm {

// Grid build (grid_build.cu).  Returns FM_* status, message in ctx->err.
int build_grid(fm_ctx* ctx, fm_scene* s, const float* d_xyz, uint32_t stride);
// Lazily built skip tables, launched on `st` (valid for every later launch
// on that stream; other streams must order after it).
int ensure_bound(fm_ctx* ctx, fm_scene* s, cudaStream_t st, float iso);
// Refine the shell boxes of a built table (once per build; a no-op otherwise).
int refine_bound(fm_ctx* ctx, fm_scene* s, cudaStream_t st);
bool bound_stale(const fm_scene* s, float iso);
int ensure_flags(fm_ctx* ctx, fm_scene* s, cudaStream_t st);
GridDev grid_dev(const fm_scene* s);

// Splat (splat.cu): depth must be a device buffer of W*H floats.
int launch_splat(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, float* d_depth, cudaStream_t st);

// Camera-derived constants of the depth pass.
struct SplatArgs {
    float V[16];
    float P00, P11, P22, P32, P23, P33;
    float R, invR;
    float twoWinv, twoHinv;
    int W, Hh;
    const float* __restrict__ hiz;  // per 8x8 tile: max depth after the sampled pass
    int hiz_w, hiz_h;
    int cull;                       // depth grows with view z: the tile test is valid
};

// One view of a batched splat.
struct SplatView {
    SplatArgs a;
    const float4* pts;
    uint64_t n;
    uint32_t* depth;  // W*H floats (as bits)
};

// Batched splat: all views in one launch per pass.  Prefix arrays have
// nviews + 1 entries: pixels, sampled particles, particles, hiz tiles.
struct SplatBatch {
    const SplatView* views;  // device
    int nviews;
    const uint64_t* pfx_px;
    const uint64_t* pfx_sample;
    const uint64_t* pfx_n;
    const uint32_t* pfx_tiles;
    float* hiz;              // all views' tiles
    uint32_t* list;          // survivors: global particle index (pfx_n[v] + i)
    unsigned int* count;     // survivor counter (zeroed by the caller)
    uint64_t tot_px, tot_sample, tot_n;
    uint32_t tot_tiles;
};
SplatArgs splat_args(const fm_scene* s, const fm_camera* cam);
constexpr int kSplatHizTile = 8;
constexpr uint64_t kSplatSample = 24;
int launch_splat_batch(fm_ctx* ctx, const SplatBatch& b, cudaStream_t st);

// March (march.cu): all pointers device pointers.
struct MarchOutDev {
    float4* pos;
    float4* nrm;
    float* depth;
    float4* col;
    const float* start_depth;
    const int2* ivl;  // proposed intervals (learned march) or null
};

// Arguments of one view.  A batch holds one per view in device memory, with
// the launch-wide fields (counters, queue, tile shape, stats, status) equal in
// all of them.
struct MarchArgs {
    GridDev g;
    KernelDev k;
    float iso, step;
    int max_steps, bisect, skip_mode;
    float cull;  // squared reach in cell units: (1 + margin)^2
    float ipv[16];
    float cam[3];
    float cdir[3];
    int W, Hh;
    int tiles_x, ntiles;   // ntiles: this view's tiles (launch argument: the launch's)
    int tw_log2;           // tile = (1 << tw_log2) x (32 >> tw_log2) pixels
    int claim;             // tiles a warp takes per atomic
    float twoWinv, twoHinv;
    const float* __restrict__ zbuf;
    const int2* __restrict__ ivl;  // proposed intervals per pixel (learned march) or null
    float4* pos;
    float4* nrm;
    float* depth;
    float4* col;
    unsigned int* tile_counter;
    unsigned int* q_tail;  // long-ray queue: entries written by the shared-stream pass
    unsigned int* q_head;  // entries taken by the long-ray pass
    float4* longq;         // 4 float4 per entry
    unsigned int q_cap;
    int cap;               // shared-stream iterations per tile before the rays left are deferred
    int defer_lanes;       // ... or once at most this many rays of the warp are active
    // regrouped second pass (launch-wide; order == null: no second pass)
    int cap2;              // its iterations before the rays left go to the warp-per-ray pass
    uint32_t* keys;        // ntiles + 1 counters of the counting sort
    uint32_t* scan_tmp;    // scan temporaries
    uint32_t* order;       // queue entries sorted by first-pass tile
    float4* longq2;        // second queue (q_cap entries)
    unsigned int* q2_tail;
    unsigned int* q2_head;
    unsigned int* grp_counter;
    unsigned long long* stats;
    unsigned int* status;
};

// Per-view fields of the march arguments (launch-wide fields left zero).
MarchArgs march_view_args(const fm_scene* s, const fm_camera* cam, const fm_march_params* p, const MarchOutDev& o,
                          const TileConfig& cfg);
// Long-ray queue entries for `pixels` rays (deferred rays are a few percent;
// a full queue only keeps rays in the first pass).
inline uint64_t long_queue_entries(uint64_t pixels, uint32_t limit = 0) {
    uint64_t q = limit ? (uint64_t)limit : pixels / 4 + 65536;
    return q < pixels ? q : pixels;
}
// Both march passes.  nviews == 0: `launch` is the single view; otherwise
// d_views / d_tile_pfx describe the batch and `launch` carries the
// launch-wide fields with ntiles = total tiles.
int launch_march_kernels(fm_ctx* ctx, const MarchArgs& launch, const MarchArgs* d_views, const uint32_t* d_tile_pfx,
                         int nviews, cudaStream_t st);
// queue: a long-ray queue of the caller's for this launch (then no regrouped
// pass), so that it can run next to another march of the context.
int launch_march(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p,
                 const MarchOutDev& o, cudaStream_t st, DevBuf* queue = nullptr);
// The anisotropic march (march.cu), warp per ray.
int launch_march_aniso(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p,
                       const fm_aniso_params* ap, const MarchOutDev& o, cudaStream_t st);
// Batched anisotropic march: per-view device blocks of aniso_view_bytes()
// (aniso_view fills one), chunks of 32 pixels with prefix pfx over the views
// (0 chunks for views without anisotropic rays); a carries the launch-wide
// counter (tile_counter, zeroed by the caller), stats and status.
size_t aniso_view_bytes();
void aniso_view(const fm_scene* s, const fm_aniso_params* ap, void* out);
int launch_march_aniso_batch(fm_ctx* ctx, const MarchArgs& a, const MarchArgs* d_views, const void* d_aviews,
                             const uint32_t* d_pfx, int nviews, uint32_t nchunks, cudaStream_t st);
// Density at n points (xyz at a stride of `stride` floats), device pointers.
int launch_density(fm_ctx* ctx, const fm_scene* s, const float* d_xyz, uint64_t n, uint32_t stride, float* d_out,
                   cudaStream_t st);

// Argument checks shared by the single and batched entry points (api.cu).
int check_camera(fm_ctx* ctx, const fm_camera* c, bool need_splat);
int check_params(fm_ctx* ctx, const fm_march_params* p);
bool grow_buf(DevBuf& b, size_t bytes);
// Exclusive prefix sum of n words (in may equal out); tmp: scan_words(n) words (grid_build.cu).
uint64_t scan_words(uint64_t n);
void scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, cudaStream_t st);
// Free the batches a context still holds (batch.cu).
void destroy_batches(fm_ctx* ctx);

// Learned proposal (proposal.cu).
int ensure_occupancy(fm_ctx* ctx, fm_scene* s, cudaStream_t st);
int launch_features(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const float* zbuf, float* feat, float* t0,
                    cudaStream_t st);
// Per-frame judge (fm_set_judge): judge_start enqueues the plain march of a
// pixel sample of a learned march whose start depths are z (on a stream of its
// own, next to the learned march); judge_finish, once both are done, compares
// the sample's hit distances with the learned ones.
int judge_start(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const fm_march_params* p, const float* z,
                cudaStream_t st);
int judge_finish(fm_ctx* ctx, const float* learned_depth, uint64_t npx, cudaStream_t st);
int launch_propose(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const fm_march_params* p, const fm_proposal* pr,
                   const float* zbuf, int2* ivl, float2* raw, cudaStream_t st);
// Batched proposal: per-view blocks (propose_view) laid out by the caller.
struct ProposeBatchDev {
    const void* views;         // nviews blocks of propose_view_bytes()
    const uint64_t* tile_pfx;  // nviews + 1: first 128-ray tile of every view
    const uint64_t* low_pfx;   // nviews + 1: first low-resolution pixel of every view
    int nviews;
    uint64_t ntiles, nlow;
    const uint64_t* blk_pfx;   // first 8x4 interval block of every view, nviews + 1
    uint64_t nblk;
    const void* weights;       // the proposal's BF16 weight image (a copy the batch owns)
    const float* bias;
};
size_t propose_view_bytes();
uint64_t propose_view_blocks(const fm_camera* cam);  // 8x4 interval blocks of a view
uint64_t propose_low_pixels(const fm_camera* cam);
// margins = {margin_lo, margin_hi, min_near} of the proposal (proposal_weights reads them)
void propose_view(const fm_scene* s, const fm_camera* cam, const fm_march_params* p, const float margins[3],
                  const float* zbuf, float* zlow, int2* ivl, void* out);
// copies the proposal's weights and bias into buffers the caller owns, and its margins
int proposal_weights(fm_ctx* ctx, const fm_proposal* pr, DevBuf& w, DevBuf& b, float margins[3], cudaStream_t st);
int launch_propose_batch(fm_ctx* ctx, const ProposeBatchDev& b, cudaStream_t st);

int set_err(fm_ctx* ctx, int code, const std::string& msg);
int cuda_err(fm_ctx* ctx, cudaError_t e, const char* what);

}  // namespace fm

#define FM_CUDA(ctx, call)                                  \
    do {                                                    \
        cudaError_t _e = (call);                            \
        if (_e != cudaSuccess) return fm::cuda_err((ctx), _e, #call); \
    } while (0)
