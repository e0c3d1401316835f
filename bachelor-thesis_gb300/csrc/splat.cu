// splat.cu -- particle sphere-splat depth (the reference's depth pass).
//
// The reference rasterises one camera-facing quad of half size R per particle
// (AdvancedRenderer.cpp:447-485) with depth.vert/depth.frag:
//   UV in [-1,1]^2, discard l2 = |UV|^2 > 1,
//   depth = proj(view_pos - R * (0, 0, cos(pi/2 * sqrt(l2)))).z / w,
// into a D32 buffer cleared to 1.0 with a LESS test (DepthRenderPass.cpp:54,179).
// The quad lies in the view-space plane z = view_z(p), so for a pixel centre
// the quad point is (ndc * z / P00, ndc * z / P11) and UV follows directly.
// Each covered pixel centre gets exactly that value, in the same FP32
// operation order as the CPU oracle, and the buffer keeps the minimum through
// an atomicMin on the float bits (depths are in [0, 1), where the uint order
// is the float order).  cos is a degree-16 Taylor polynomial (coefficients
// 1/(2k)! as exact float literals), identical in the oracle.
//
// A warp splats one particle: its lanes walk the disc's pixel box 32 pixels
// at a time.  Three passes keep the work near the visible surface without
// changing the result (the buffer is a minimum, so leaving out a particle that
// cannot lower any pixel is exact):
//   1. every 24th particle (in cell order) is splatted: the discs, about five
//      particle spacings wide, already form a nearly opaque cover of the front
//      surface;
//   2. a max-depth tile level (8x8 pixels) is built from the buffer, and every
//      other particle is tested against it: it is kept only if some tile
//      under its disc holds a depth above the nearest depth the disc can have
//      (disc_min_bits: the depth at view z - R, lowered for rounding); the buffer
//      after pass 1 is >= the final one, so no fragment that would win a
//      pixel is dropped;
//   3. the kept particles are splatted.
// Within a disc, a pixel whose buffer already holds a depth at or below the
// disc's minimum is skipped before its fragment is computed.
// Memory: 16 B per particle, 4 B read (+ atomic) per covered pixel of a
// splatted particle, 4 B per tile.

#include <cuda_runtime.h>

#include "fm_internal.cuh"

namespace fm {
namespace {

constexpr int kHizTile = kSplatHizTile;
constexpr uint64_t kSample = kSplatSample;
constexpr int kThreads = 256;

__device__ __forceinline__ float cos_poly(float t) {
    float x = t * t;
    float p = 0x1.ae7f3ep-45f;
    p = p * x - 0x1.93974ap-37f;
    p = p * x + 0x1.1eed8ep-29f;
    p = p * x - 0x1.27e4fcp-22f;
    p = p * x + 0x1.a01a02p-16f;
    p = p * x - 0x1.6c16c2p-10f;
    p = p * x + 0x1.555556p-5f;
    p = p * x - 0x1.0p-1f;
    p = p * x + 1.0f;
    return p;
}

__global__ void k_fill(uint32_t* __restrict__ d, uint64_t n, uint32_t v) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) d[i] = v;
}

// View-space centre and conservative pixel box of a particle's disc.
// Returns false when the disc is not entirely in front of the camera or off screen.
__device__ __forceinline__ bool disc_box(const SplatArgs& a, const float4& q, float& cx, float& cy, float& cz, int& x0,
                                         int& x1, int& y0, int& y1) {
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float add0 = a.V[0 * 4 + r] * q.x + a.V[1 * 4 + r] * q.y;
        float add1 = a.V[2 * 4 + r] * q.z + a.V[3 * 4 + r] * 1.0f;
        c[r] = add0 + add1;
    }
    cx = c[0] / c[3];
    cy = c[1] / c[3];
    cz = c[2] / c[3];
    const float R = a.R;
    if (!(cz - R > 0.0f)) return false;
    float nx0 = a.P00 * (cx - R) / cz, nx1 = a.P00 * (cx + R) / cz;
    float ny0 = a.P11 * (cy - R) / cz, ny1 = a.P11 * (cy + R) / cz;
    float xa = fminf(nx0, nx1), xb = fmaxf(nx0, nx1);
    float ya = fminf(ny0, ny1), yb = fmaxf(ny0, ny1);
    float fx0 = floorf((xa + 1.0f) * 0.5f * (float)a.W - 0.5f) - 1.0f;
    float fx1 = ceilf((xb + 1.0f) * 0.5f * (float)a.W - 0.5f) + 1.0f;
    float fy0 = floorf((ya + 1.0f) * 0.5f * (float)a.Hh - 0.5f) - 1.0f;
    float fy1 = ceilf((yb + 1.0f) * 0.5f * (float)a.Hh - 0.5f) + 1.0f;
    if (fx1 < 0.0f || fy1 < 0.0f || fx0 > (float)(a.W - 1) || fy0 > (float)(a.Hh - 1)) return false;
    x0 = max(0, (int)fmaxf(fx0, -1.0f));
    x1 = min(a.W - 1, (int)fminf(fx1, (float)a.W));
    y0 = max(0, (int)fmaxf(fy0, -1.0f));
    y1 = min(a.Hh - 1, (int)fminf(fy1, (float)a.Hh));
    return true;
}

// The disc's quad coordinates of pixel column x (uu) and row y (vv): the
// view-plane point of the pixel centre relative to the particle, in radii.
__device__ __forceinline__ float disc_u(const SplatArgs& a, float cx, float cz, int x) {
    float nx = ((float)x + 0.5f) * a.twoWinv - 1.0f;
    float vx = (nx * cz) / a.P00;
    return (vx - cx) * a.invR;
}
__device__ __forceinline__ float disc_v(const SplatArgs& a, float cy, float cz, int y) {
    float ny = ((float)y + 0.5f) * a.twoHinv - 1.0f;
    float vy = (ny * cz) / a.P11;
    return (vy - cy) * a.invR;
}

// Bits of a depth no fragment of a disc at view z = cz can go below, or 0
// when there is no such bound.  Every fragment's view z, cz - R * cos(...)
// with the cosine <= 1, rounds to >= cz - R; the projected depth
// (P22 z + P32) / (P23 z + P33) grows with z when P22 P33 - P23 P32 > 0 and
// the denominator is positive and non-decreasing.  The bound is the depth at
// cz - R lowered by 64 ulps, taken only where the projection's two sums cancel
// little (|terms| <= 4 |sum|): then the rounding of a depth is a few ulps and
// two depths in order cannot come out more than ~40 ulps out of order.
__device__ __forceinline__ uint32_t disc_min_bits(const SplatArgs& a, float cz) {
    const float zv = cz - a.R;
    const float num = a.P22 * zv, den = a.P23 * zv;
    const float A = num + a.P32, B = den + a.P33;
    if (!(a.P22 * a.P33 - a.P23 * a.P32 > 0.0f) || !(a.P23 >= 0.0f) || !(A > 0.0f) || !(B > 0.0f) ||
        !(fabsf(num) + fabsf(a.P32) <= 4.0f * A) || !(fabsf(den) + fabsf(a.P33) <= 4.0f * B))
        return 0u;
    const uint32_t db = __float_as_uint(A / B);
    return db > 64u ? db - 64u : 0u;
}

// One pixel centre of a disc (depth.frag:19-34 restated), from its quad
// coordinates.  A pixel whose buffer already holds a depth at or below the
// disc's minimum (dmin) cannot be lowered and is left alone.
__device__ __forceinline__ void splat_uv(const SplatArgs& a, float cz, float uu, float vv, int x, int y,
                                         uint32_t dmin, uint32_t* __restrict__ depth) {
    const float R = a.R;
    float l2 = uu * uu + vv * vv;
    if (l2 > 1.0f) return;
    uint32_t* dst = depth + (uint64_t)y * a.W + x;
    // plain (possibly stale) read: the buffer only decreases, so a stale value
    // is >= the current one and skipping on it is safe
    const uint32_t cur = *dst;
    if (dmin >= cur) return;
    float off = cos_poly(1.57079632679f * sqrtf(l2));
    float zv = cz - R * off;
    float d = (a.P22 * zv + a.P32) / (a.P23 * zv + a.P33);
    if (!(d >= 0.0f && d < 1.0f)) return;
    d = d + 0.0f;
    const uint32_t bits = __float_as_uint(d);
    if (bits < cur) atomicMin(dst, bits);
}

// The whole warp splats one disc: lane l starts at box pixel l and advances
// 32 pixels per step.  The quad coordinates depend on the column or on the row
// only: for boxes up to kBox pixels a side the warp computes them once per
// column and row into shared memory (the same operations, so the same bits)
// and every pixel reads two of them.
constexpr int kBox = 128;

__device__ __forceinline__ void splat_disc_warp(const SplatArgs& a, float cx, float cy, float cz, int x0, int x1,
                                                int y0, int y1, int lane, uint32_t* __restrict__ depth) {
    __shared__ float s_u[kThreads / 32][kBox], s_v[kThreads / 32][kBox];
    const int bw = x1 - x0 + 1, bh = y1 - y0 + 1;
    const uint32_t dmin = disc_min_bits(a, cz);
    int x = x0 + lane, y = y0;
    while (x > x1) { x -= bw; ++y; }
    if (bw <= kBox && bh <= kBox) {
        float* su = s_u[threadIdx.x >> 5];
        float* sv = s_v[threadIdx.x >> 5];
        __syncwarp();  // the previous disc's reads are done
        for (int i = lane; i < bw; i += 32) su[i] = disc_u(a, cx, cz, x0 + i);
        for (int i = lane; i < bh; i += 32) sv[i] = disc_v(a, cy, cz, y0 + i);
        __syncwarp();
        while (y <= y1) {
            splat_uv(a, cz, su[x - x0], sv[y - y0], x, y, dmin, depth);
            x += 32;
            while (x > x1) { x -= bw; ++y; }
        }
        return;
    }
    while (y <= y1) {
        splat_uv(a, cz, disc_u(a, cx, cz, x), disc_v(a, cy, cz, y), x, y, dmin, depth);
        x += 32;
        while (x > x1) { x -= bw; ++y; }
    }
}

// Pass 1 (stride = kSample) or the only pass (stride = 1): warp w splats
// particle w * stride, for every warp of a persistent grid.
__global__ void __launch_bounds__(kThreads) k_splat_warp(const float4* __restrict__ pts, uint64_t n, uint64_t stride,
                                                        SplatArgs a, uint32_t* __restrict__ depth) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (kThreads / 32);
    for (uint64_t w = (blockIdx.x * (uint64_t)kThreads + threadIdx.x) / 32; w * stride < n; w += warps) {
        const float4 q = pts[w * stride];
        float cx, cy, cz;
        int x0, x1, y0, y1;
        if (!disc_box(a, q, cx, cy, cz, x0, x1, y0, y1)) continue;
        splat_disc_warp(a, cx, cy, cz, x0, x1, y0, y1, lane, depth);
    }
}

// Max depth of each 8x8 tile of the buffer.
__global__ void k_hiz(const float* __restrict__ depth, int W, int Hh, int tw, int th, float* __restrict__ hiz) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tw * th) return;
    const int tx = t % tw, ty = t / tw;
    float m = 0.0f;
    for (int y = ty * kHizTile; y < min(ty * kHizTile + kHizTile, Hh); ++y)
        for (int x = tx * kHizTile; x < min(tx * kHizTile + kHizTile, W); ++x) m = fmaxf(m, depth[(uint64_t)y * W + x]);
    hiz[t] = m;
}

// Cull test of pass 2: true when the disc of q may still lower a pixel.
__device__ __forceinline__ bool cull_keep(const SplatArgs& a, const float4& q) {
    float cx, cy, cz;
    int x0, x1, y0, y1;
    if (!disc_box(a, q, cx, cy, cz, x0, x1, y0, y1)) return false;
    if (!a.cull) return true;
    const float dmin = __uint_as_float(disc_min_bits(a, cz));
    for (int ty = y0 / kHizTile; ty <= y1 / kHizTile; ++ty)
        for (int tx = x0 / kHizTile; tx <= x1 / kHizTile; ++tx)
            if (a.hiz[ty * a.hiz_w + tx] > dmin) return true;
    return false;
}

// Append the kept entries of a warp to list (one atomic per warp).
__device__ __forceinline__ void append(bool keep, uint32_t value, uint32_t* __restrict__ list,
                                       unsigned int* __restrict__ count) {
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    unsigned base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) list[base + __popc(m & ((1u << lane) - 1u))] = value;
}

// Pass 2: the particles pass 1 left out, tested against the tile maxima; the
// ones that may still lower a pixel are appended to `list`.
__global__ void __launch_bounds__(kThreads) k_splat_cull(const float4* __restrict__ pts, uint64_t n, SplatArgs a,
                                                        uint32_t* __restrict__ list, unsigned int* __restrict__ count) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const bool keep = i < n && (i % kSample) != 0 && cull_keep(a, pts[i]);
    append(keep, (uint32_t)i, list, count);
}

// Pass 3: warp per kept particle.
__global__ void __launch_bounds__(kThreads) k_splat_list(const float4* __restrict__ pts,
                                                        const uint32_t* __restrict__ list,
                                                        const unsigned int* __restrict__ count, SplatArgs a,
                                                        uint32_t* __restrict__ depth) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (kThreads / 32);
    const uint64_t total = *count;
    for (uint64_t w = (blockIdx.x * (uint64_t)kThreads + threadIdx.x) / 32; w < total; w += warps) {
        const float4 q = pts[list[w]];
        float cx, cy, cz;
        int x0, x1, y0, y1;
        if (!disc_box(a, q, cx, cy, cz, x0, x1, y0, y1)) continue;
        splat_disc_warp(a, cx, cy, cz, x0, x1, y0, y1, lane, depth);
    }
}

// ---- batched passes: one launch per pass over the units of all views --------

// The largest v with pfx[v] <= u (pfx ascending, pfx[0] = 0).
template <typename T>
__device__ __forceinline__ int find_view(const T* __restrict__ pfx, int nviews, T u) {
    int lo = 0, hi = nviews - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pfx[mid] <= u) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__global__ void k_fill_b(SplatBatch b) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= b.tot_px) return;
    const int v = find_view(b.pfx_px, b.nviews, i);
    b.views[v].depth[i - b.pfx_px[v]] = 0x3f800000u;
}

// Pass 1: warp per sampled particle (every kSample-th of each view).
__global__ void __launch_bounds__(kThreads) k_splat_warp_b(SplatBatch b) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (kThreads / 32);
    for (uint64_t w = (blockIdx.x * (uint64_t)kThreads + threadIdx.x) / 32; w < b.tot_sample; w += warps) {
        const int v = find_view(b.pfx_sample, b.nviews, w);
        const SplatView& sv = b.views[v];
        const float4 q = sv.pts[(w - b.pfx_sample[v]) * kSample];
        float cx, cy, cz;
        int x0, x1, y0, y1;
        if (!disc_box(sv.a, q, cx, cy, cz, x0, x1, y0, y1)) continue;
        splat_disc_warp(sv.a, cx, cy, cz, x0, x1, y0, y1, lane, sv.depth);
    }
}

__global__ void k_hiz_b(SplatBatch b) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.tot_tiles) return;
    const int v = find_view(b.pfx_tiles, b.nviews, t);
    const SplatView& sv = b.views[v];
    const int tl = (int)(t - b.pfx_tiles[v]);
    const int tx = tl % sv.a.hiz_w, ty = tl / sv.a.hiz_w;
    const float* depth = (const float*)sv.depth;
    float m = 0.0f;
    for (int y = ty * kHizTile; y < min(ty * kHizTile + kHizTile, sv.a.Hh); ++y)
        for (int x = tx * kHizTile; x < min(tx * kHizTile + kHizTile, sv.a.W); ++x)
            m = fmaxf(m, depth[(uint64_t)y * sv.a.W + x]);
    b.hiz[t] = m;
}

__global__ void __launch_bounds__(kThreads) k_splat_cull_b(SplatBatch b) {
    const uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    bool keep = false;
    if (g < b.tot_n) {
        const int v = find_view(b.pfx_n, b.nviews, g);
        const SplatView& sv = b.views[v];
        const uint64_t i = g - b.pfx_n[v];
        keep = (i % kSample) != 0 && cull_keep(sv.a, sv.pts[i]);
    }
    append(keep, (uint32_t)g, b.list, b.count);
}

__global__ void __launch_bounds__(kThreads) k_splat_list_b(SplatBatch b) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (kThreads / 32);
    const uint64_t total = *b.count;
    for (uint64_t w = (blockIdx.x * (uint64_t)kThreads + threadIdx.x) / 32; w < total; w += warps) {
        const uint64_t g = b.list[w];
        const int v = find_view(b.pfx_n, b.nviews, g);
        const SplatView& sv = b.views[v];
        const float4 q = sv.pts[g - b.pfx_n[v]];
        float cx, cy, cz;
        int x0, x1, y0, y1;
        if (!disc_box(sv.a, q, cx, cy, cz, x0, x1, y0, y1)) continue;
        splat_disc_warp(sv.a, cx, cy, cz, x0, x1, y0, y1, lane, sv.depth);
    }
}

}  // namespace

bool grow_buf(DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) return false;
    b.bytes = bytes;
    return true;
}

SplatArgs splat_args(const fm_scene* s, const fm_camera* cam) {
    SplatArgs a;
    for (int i = 0; i < 16; ++i) a.V[i] = cam->view[i];
    a.P00 = cam->proj[0];
    a.P11 = cam->proj[5];
    a.P22 = cam->proj[10];
    a.P32 = cam->proj[14];
    a.P23 = cam->proj[11];
    a.P33 = cam->proj[15];
    a.R = s->support;
    a.invR = 1.0f / s->support;
    a.W = cam->width;
    a.Hh = cam->height;
    a.twoWinv = 2.0f / (float)cam->width;
    a.twoHinv = 2.0f / (float)cam->height;
    a.hiz = nullptr;
    a.hiz_w = (cam->width + kHizTile - 1) / kHizTile;
    a.hiz_h = (cam->height + kHizTile - 1) / kHizTile;
    // the culling test needs depth to grow with view z: d(z) = (P22 z + P32) / (P23 z + P33)
    a.cull = ((a.P22 * a.P33 - a.P32 * a.P23) > 0.0f && a.P23 > 0.0f && a.P33 >= 0.0f) ? 1 : 0;
    return a;
}

int launch_splat(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, float* d_depth, cudaStream_t st) {
    SplatArgs a = splat_args(s, cam);
    const uint64_t npx = (uint64_t)cam->width * cam->height;
    k_fill<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>((uint32_t*)d_depth, npx, 0x3f800000u);
    if (s->n == 0) return FM_OK;
    const unsigned persist = (unsigned)ctx->sm_count * 8;  // 64 warps per SM
    if (!a.cull) {
        k_splat_warp<<<persist, kThreads, 0, st>>>(s->d_pts, s->n, 1, a, (uint32_t*)d_depth);
        FM_CUDA(ctx, cudaGetLastError());
        return FM_OK;
    }
    const size_t hiz_bytes = (size_t)a.hiz_w * a.hiz_h * sizeof(float);
    if (ctx->hiz.bytes < hiz_bytes || ctx->splat_list.bytes < s->n * sizeof(uint32_t)) {
        FM_CUDA(ctx, cudaStreamSynchronize(st));  // old buffers may still be in use on this stream
        if (!grow_buf(ctx->hiz, hiz_bytes) || !grow_buf(ctx->splat_list, s->n * sizeof(uint32_t)))
            return set_err(ctx, FM_ERR_OOM, "splat buffer allocation failed");
    }
    a.hiz = (const float*)ctx->hiz.p;
    unsigned int* count = ctx->d_work + (ctx->work_slot++ % kWorkSlots) * 32;
    FM_CUDA(ctx, cudaMemsetAsync(count, 0, sizeof(unsigned int), st));
    k_splat_warp<<<persist, kThreads, 0, st>>>(s->d_pts, s->n, kSample, a, (uint32_t*)d_depth);
    const int tiles = a.hiz_w * a.hiz_h;
    k_hiz<<<(tiles + 255) / 256, 256, 0, st>>>(d_depth, a.W, a.Hh, a.hiz_w, a.hiz_h, (float*)ctx->hiz.p);
    k_splat_cull<<<(unsigned)((s->n + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        s->d_pts, s->n, a, (uint32_t*)ctx->splat_list.p, count);
    k_splat_list<<<persist, kThreads, 0, st>>>(s->d_pts, (const uint32_t*)ctx->splat_list.p, count, a,
                                               (uint32_t*)d_depth);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

// Batched depth pass: fill, sampled pass, tile maxima, cull, survivors; one
// launch each for all views.  Views whose projection does not allow the tile
// test keep all their particles in the list (the result is the same).
int launch_splat_batch(fm_ctx* ctx, const SplatBatch& b, cudaStream_t st) {
    if (b.tot_px) k_fill_b<<<(unsigned)((b.tot_px + 255) / 256), 256, 0, st>>>(b);
    if (b.tot_n == 0) return FM_OK;
    const unsigned persist = (unsigned)ctx->sm_count * 8;
    k_splat_warp_b<<<persist, kThreads, 0, st>>>(b);
    if (b.tot_tiles) k_hiz_b<<<(b.tot_tiles + 255) / 256, 256, 0, st>>>(b);
    k_splat_cull_b<<<(unsigned)((b.tot_n + kThreads - 1) / kThreads), kThreads, 0, st>>>(b);
    k_splat_list_b<<<persist, kThreads, 0, st>>>(b);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace fm
