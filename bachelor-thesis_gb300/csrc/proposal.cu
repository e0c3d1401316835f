// proposal.cu -- learned hit-interval proposal for the march.
//
// No counterpart in the reference, whose march starts every ray at its splat
// depth and steps until the first density >= iso (RayMarcher.cpp:276-343).
// Here a small MLP looks at each ray before the march and proposes an interval
// [near, far] of the ray in which the first crossing should lie; the exact
// march (march.cu, LEARNED) then evaluates only the samples of the plain
// march's own sample lattice inside that interval, and restarts as the full
// plain march when the interval holds no crossing or starts inside the fluid.
// A hit mask therefore never changes; a depth can only differ when the fluid
// is crossed before `near` (the judge, k_judge, counts those pixels).
//
// Pieces:
//   occupancy   64^3 FP16 grid over the scene box: SPH density at the voxel
//               centres over the kernel peak W(0) (iso / W(0) is ~30 for the
//               sloshing family at half rest density)
//   features    per ray (32 slots, 23 used): 16 trilinear occupancy samples at
//               0.25 H .. 7.75 H past the ray start, the 1/8-resolution splat
//               depth offset, the ray direction, the start point in the box
//   inference   k_propose: 128 rays per CTA tile, the three layers as
//               tcgen05.mma kind::f16 (BF16 operands from shared memory,
//               FP32 accumulators in tensor memory), bias + GELU epilogues
//               read back with tcgen05.ld
//   training    FP32 SIMT kernels: forward, backward (pinball loss on the
//               near / far outputs), gradient reduction, Adam
//   judge       k_judge: hit-mask mismatches and depth errors of a march
//               against a reference march
//
// MLP parameters, FP32 blob of kProposalParams floats:
//   W1[64][32], b1[64], W2[64][64], b2[64], W3[2][64], b3[2]
// (W[out][in]); outputs are (near, far) in support radii past the ray start.

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "fm_internal.cuh"

struct fm_proposal {
    fm_ctx* ctx = nullptr;
    void* d_weights = nullptr;  // BF16 W1 | W2 | W3 in k_propose's shared-memory image
    float* d_bias = nullptr;    // b1 | b2 | b3
    float margin_lo = 0.0f, margin_hi = 0.0f;
    float min_near = 0.0f;  // intervals starting closer than this (support radii) are not used
};

struct fm_trainer {
    fm_ctx* ctx = nullptr;
    float* d_p = nullptr;  // parameters, gradient, Adam moments: 4 x kProposalParams
    fm::DevBuf work;       // activations of the largest batch
    uint32_t cap = 0;
    int steps = 0;
};

namespace fm {
namespace {

constexpr int kOcc = kProposalOcc;   // occupancy grid resolution
constexpr int kF = kProposalFeatures;
constexpr int kH = 64;               // hidden width
constexpr int kO = 2;
constexpr int kRows = 128;           // rays per tensor-core tile (MMA M)
constexpr int kN3 = 16;              // last layer padded to the smallest MMA N
constexpr int kLow = 8;              // low-resolution depth factor
constexpr int oW1 = 0, oB1 = oW1 + kH * kF, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH, oB3 = oW3 + kO * kH;
static_assert(oB3 + kO == kProposalParams, "parameter blob layout");

// shared-memory image of k_propose (bytes)
constexpr uint32_t kSmA1 = 0;                    // 128 x 32 BF16 features
constexpr uint32_t kSmA2 = kSmA1 + kRows * kF * 2;  // 128 x 64 BF16 hidden activations
constexpr uint32_t kSmW1 = kSmA2 + kRows * kH * 2;  // 64 x 32
constexpr uint32_t kSmW2 = kSmW1 + kH * kF * 2;     // 64 x 64
constexpr uint32_t kSmW3 = kSmW2 + kH * kH * 2;     // 16 x 64
constexpr uint32_t kWeightBytes = (kH * kF + kH * kH + kN3 * kH) * 2;  // 14336
constexpr uint32_t kSmBias = kSmW3 + kN3 * kH * 2;  // 130 floats
constexpr uint32_t kSmBar = kSmBias + 544;          // mbarrier (8 B)
constexpr uint32_t kSmTmem = kSmBar + 8;            // TMEM base address
constexpr uint32_t kSmUsed = kSmTmem + 8;
// Requested dynamic shared memory: more than a sixth of the SM's 228 KB, so
// at most 5 CTAs share an SM and their 5 x 64 TMEM columns always fit in 512.
// The three layers' accumulators share the same 64 columns: a layer's MMA is
// issued only after the previous epilogue has read them back.
constexpr uint32_t kSmRequest = 40 * 1024;
constexpr uint32_t kTmemCols = 64;
constexpr int kCtasPerSm = 5;          // persistent grid: CTAs resident per SM
constexpr uint32_t kWaitLimit = 1u << 22;  // mbarrier polls before giving up
static_assert(kSmUsed <= kSmRequest, "shared memory image");

// Byte offset of element (row, k) of a K-major tile with K columns in the
// canonical no-swizzle layout: 8x8 core matrices of 128 contiguous bytes
// (8 rows of 16 B), K-adjacent core matrices 128 B apart (leading byte
// offset), 8-row groups (K/8) * 128 B apart (stride byte offset).
__host__ __device__ __forceinline__ uint32_t canon_off(int row, int k, int K) {
    return (uint32_t)(((row >> 3) * (K >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// ---- occupancy ----------------------------------------------------------------

// Density at every voxel centre, in units of the kernel's peak W(0): an
// "effective neighbour count" that does not depend on the support radius.
// Thread per voxel, summing the 27 grid cells around the centre.
__global__ void k_occ_density(const GridDev g, const KernelDev k, float ox, float oy, float oz, float vx, float vy,
                              float vz, __half* __restrict__ occ) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= kOcc * kOcc * kOcc) return;
    const int ix = v % kOcc, iy = (v / kOcc) % kOcc, iz = v / (kOcc * kOcc);
    const float cx = ox + ((float)ix + 0.5f) * vx, cy = oy + ((float)iy + 0.5f) * vy, cz = oz + ((float)iz + 0.5f) * vz;
    int c[3];
    float rho = 0.0f;
    if (sample_cell(g, cx, cy, cz, c[0], c[1], c[2])) {
        for (int z = max(c[2] - 1, 0); z <= min(c[2] + 1, g.dims[2] - 1); ++z)
            for (int y = max(c[1] - 1, 0); y <= min(c[1] + 1, g.dims[1] - 1); ++y) {
                const int x0 = max(c[0] - 1, 0), x1 = min(c[0] + 1, g.dims[0] - 1);
                if (x0 > x1) continue;
                const uint32_t row = ((uint32_t)z * (uint32_t)g.dims[1] + (uint32_t)y) * (uint32_t)g.dims[0];
                const uint32_t b = __ldg(g.sub + 8u * (row + (uint32_t)x0)), e = __ldg(g.sub + 8u * (row + (uint32_t)x1) + 8u);
                for (uint32_t j = b; j < e; ++j) {
                    const float4 q = __ldg(g.pts + j);
                    const float rx = q.x - cx, ry = q.y - cy, rz = q.z - cz;
                    const float d = dot3(rx, ry, rz, rx, ry, rz);
                    if (d < k.h2) rho = rho + w_in(k, d);
                }
            }
    }
    occ[v] = __float2half(fminf(rho / k.sig, 60000.0f));
}

// Minimum depth of each kLow x kLow block.
__global__ void k_lowres(const float* __restrict__ z, int W, int Hh, int lw, int lh, float* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lw * lh) return;
    const int bx = t % lw, by = t / lw;
    float m = 1.0f;
    for (int y = by * kLow; y < min(by * kLow + kLow, Hh); ++y)
        for (int x = bx * kLow; x < min(bx * kLow + kLow, W); ++x) m = fminf(m, z[(uint64_t)y * W + x]);
    out[t] = m;
}

// ---- features -------------------------------------------------------------------


struct FeatArgs {
    float ipv[16];
    float cam[3];
    float twoWinv, twoHinv;
    int W, Hh, lw;
    const float* __restrict__ zbuf;
    const float* __restrict__ zlow;
    const __half* __restrict__ occ;
    float omin[3], oinv[3];  // occupancy box and voxels per unit length
    float bmin[3], binv[3];  // scene box and 1 / extent
    float H, invH;
};

__device__ __forceinline__ void unproject(const FeatArgs& a, int px, int py, float z, float p[3]) {
    const float cx = (float)px * a.twoWinv - 1.0f, cy = (float)py * a.twoHinv - 1.0f;
    float w[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) w[r] = (a.ipv[r] * cx + a.ipv[4 + r] * cy) + (a.ipv[8 + r] * z + a.ipv[12 + r]);
    p[0] = w[0] / w[3];
    p[1] = w[1] / w[3];
    p[2] = w[2] / w[3];
}

// Trilinear occupancy at x (voxel centres at (i + 0.5) / oinv; outside: 0).
__device__ __forceinline__ float occ_at(const FeatArgs& a, float x, float y, float z) {
    const float fx = (x - a.omin[0]) * a.oinv[0] - 0.5f;
    const float fy = (y - a.omin[1]) * a.oinv[1] - 0.5f;
    const float fz = (z - a.omin[2]) * a.oinv[2] - 0.5f;
    if (!(fx > -1.0f && fy > -1.0f && fz > -1.0f && fx < (float)kOcc && fy < (float)kOcc && fz < (float)kOcc))
        return 0.0f;
    const int x0 = (int)floorf(fx), y0 = (int)floorf(fy), z0 = (int)floorf(fz);
    const float tx = fx - (float)x0, ty = fy - (float)y0, tz = fz - (float)z0;
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int xi = x0 + (c & 1), yi = y0 + ((c >> 1) & 1), zi = z0 + (c >> 2);
        if (xi < 0 || yi < 0 || zi < 0 || xi >= kOcc || yi >= kOcc || zi >= kOcc) continue;
        const float w = ((c & 1) ? tx : 1.0f - tx) * (((c >> 1) & 1) ? ty : 1.0f - ty) * ((c >> 2) ? tz : 1.0f - tz);
        s += w * __half2float(a.occ[(zi * kOcc + yi) * kOcc + xi]);
    }
    return s;
}

// Features of pixel (px, py); false when its ray does not start (no particle).
__device__ __forceinline__ bool ray_features(const FeatArgs& a, int px, int py, float f[kF], float& t0) {
    const float z = a.zbuf[(uint64_t)py * a.W + px];
#pragma unroll
    for (int j = 0; j < kF; ++j) f[j] = 0.0f;
    t0 = 0.0f;
    if (z == 1.0f) return false;
    float p0[3];
    unproject(a, px, py, z, p0);
    const float dx = p0[0] - a.cam[0], dy = p0[1] - a.cam[1], dz = p0[2] - a.cam[2];
    t0 = sqrtf(dx * dx + dy * dy + dz * dz);
    const float inv = 1.0f / fmaxf(t0, 1e-30f);
    const float d[3] = {dx * inv, dy * inv, dz * inv};
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const float t = a.H * (0.25f + 0.5f * (float)j);
        f[j] = occ_at(a, p0[0] + d[0] * t, p0[1] + d[1] * t, p0[2] + d[2] * t);
    }
    const float zc = a.zlow[(py / kLow) * a.lw + px / kLow];
    float pc[3];
    unproject(a, px, py, zc, pc);
    const float cx = pc[0] - a.cam[0], cy = pc[1] - a.cam[1], cz = pc[2] - a.cam[2];
    const float tc = sqrtf(cx * cx + cy * cy + cz * cz);
    f[16] = 0.25f * fmaxf(fminf((tc - t0) * a.invH, 0.0f), -16.0f);
    f[17] = d[0];
    f[18] = d[1];
    f[19] = d[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) f[20 + k] = (p0[k] - a.bmin[k]) * a.binv[k];
    return true;
}

__global__ void k_features(const FeatArgs a, float* __restrict__ feat, float* __restrict__ t0) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)a.W * a.Hh) return;
    float f[kF], t;
    ray_features(a, (int)(i % a.W), (int)(i / a.W), f, t);
#pragma unroll
    for (int j = 0; j < kF; j += 4) *(float4*)(feat + i * kF + j) = make_float4(f[j], f[j + 1], f[j + 2], f[j + 3]);
    if (t0) t0[i] = t;
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

struct IvlArgs {
    float H, step;
    int max_steps;
    float margin_lo, margin_hi, min_near;
};

// (near, far) in support radii -> march samples (ks, kf): evaluate ks+1 .. kf.
// (0, -1): no usable interval, the ray runs the full march.
__device__ __forceinline__ int2 to_interval(const IvlArgs& v, float y0, float y1) {
    const float near = y0 - v.margin_lo, far = y1 + v.margin_hi;
    if (!(near == near) || !(far == far) || !(far > near) || !(far > 0.0f) || !(near >= v.min_near))
        return make_int2(0, -1);
    const float s0 = fmaxf(near, 0.0f) * v.H / v.step, s1 = far * v.H / v.step;
    if (!(s0 < 1.0e6f)) return make_int2(0, -1);
    const int ks = (int)floorf(s0);
    const int kf = (int)fminf(ceilf(fminf(s1, 1.0e6f)) + 1.0f, (float)v.max_steps);
    if (ks < 1 || kf <= ks) return make_int2(0, -1);
    return make_int2(ks, kf);
}

// ---- tensor-core inference ----------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// tcgen05 shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t mdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version (bits 46-48 = 0b001)
    return d;                // base offset 0, absolute LBO mode, layout SWIZZLE_NONE
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t n) {
    return (1u << 4)              // D format F32
           | (1u << 7)            // A format BF16
           | (1u << 10)           // B format BF16
           | ((n >> 3) << 17)     // N / 8
           | ((128u >> 4) << 24); // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, uint32_t limit = kWaitLimit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
           ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

// Store 8 consecutive K values of row `row` (k0 multiple of 8) as BF16.
__device__ __forceinline__ void store8(uint8_t* tile, int row, int k0, int K, const float* v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *(uint4*)(tile + canon_off(row, k0, K)) = q;
}

// One view of the proposal: its features, interval settings and outputs.
struct ProposeView {
    FeatArgs f;
    IvlArgs v;
    int2* __restrict__ ivl;
    float2* __restrict__ raw;             // optional (near, far) outputs
    uint64_t npx;
};

struct ProposeArgs {
    ProposeView one;                      // single view
    const ProposeView* __restrict__ views;  // batch: per-view blocks (device)
    const uint64_t* __restrict__ tile_pfx;  // batch: first tile of every view, nviews + 1
    int nviews;
    uint64_t ntiles;                      // tiles of 128 rays over all views
    const uint8_t* __restrict__ weights;  // kWeightBytes: W1, W2, W3 in the shared-memory image
    const float* __restrict__ bias;       // b1[64], b2[64], b3[2]
    unsigned int* status;
};

// Hidden layer epilogue: TMEM columns [c0, c0 + 64) of this row -> bias + GELU -> BF16 A tile.
// One copy for both hidden layers, a loop over four groups of 16 columns: the
// kernel's code stays small (instruction fetch was its top stall).
__device__ __noinline__ void hidden_epilogue(uint32_t tmem_row, uint32_t c0, const float* bias, uint8_t* a2,
                                             int row) {
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        float v[16];
        tmem_ld16(tmem_row + c0 + 16 * q, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = gelu(v[i] + bias[16 * q + i]);
        store8(a2, row, 16 * q, kH, v);
        store8(a2, row, 16 * q + 8, kH, v + 8);
    }
}

// Shared-memory and tensor-memory state of a k_propose CTA.
struct ProposeCta {
    uint8_t* sm;
    uint32_t sbase, bar, tmem, tmem_row;
};

// Tile `lt` (128 rays) of view pv: features -> three MMA layers -> intervals.
// Uniform over the CTA; false when an MMA did not complete in time.
__device__ __forceinline__ bool propose_tile(const ProposeView& pv, uint64_t lt, const ProposeCta& c, uint32_t& phase) {
    const int tid = threadIdx.x;
    const float* bias = (const float*)(c.sm + kSmBias);
    uint8_t* a1 = c.sm + kSmA1;
    uint8_t* a2 = c.sm + kSmA2;
    const uint32_t a1s = c.sbase + kSmA1, a2s = c.sbase + kSmA2;
    const uint32_t w1s = c.sbase + kSmW1, w2s = c.sbase + kSmW2, w3s = c.sbase + kSmW3;
    const uint64_t pix = lt * kRows + (uint64_t)tid;
    float f[kF], t0 = 0.0f;
    bool has = false;
    if (pix < pv.npx) has = ray_features(pv.f, (int)(pix % pv.f.W), (int)(pix / pv.f.W), f, t0);
    else {
#pragma unroll
        for (int j = 0; j < kF; ++j) f[j] = 0.0f;
    }
    // a tile without any ray needs no network
    if (!__syncthreads_or(has)) {
        if (pix < pv.npx) {
            pv.ivl[pix] = make_int2(0, -1);
            if (pv.raw) pv.raw[pix] = make_float2(0.0f, 0.0f);
        }
        return true;
    }
#pragma unroll
    for (int k = 0; k < kF; k += 8) store8(a1, tid, k, kF, f + k);
    // layer 1: D[:, 0:64) = A1 (128 x 32) * W1^T
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    if (tid == 0) {
#pragma unroll
        for (int kk = 0; kk < kF / 16; ++kk)
            mma_bf16(c.tmem, mdesc(a1s + 256 * kk, 128, (kF / 8) * 128), mdesc(w1s + 256 * kk, 128, (kF / 8) * 128),
                     idesc_bf16(kH), kk > 0 ? 1u : 0u);
        mma_commit(c.bar);
    }
    bool ok = __syncthreads_and(mbar_wait(c.bar, phase));
    phase ^= 1;
    if (!ok) return false;
    tc_after();
    hidden_epilogue(c.tmem_row, 0, bias, a2, tid);
    // layer 2: D[:, 0:64) = H1 (128 x 64) * W2^T (epilogue 1 has read layer 1's D)
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    if (tid == 0) {
#pragma unroll
        for (int kk = 0; kk < kH / 16; ++kk)
            mma_bf16(c.tmem, mdesc(a2s + 256 * kk, 128, (kH / 8) * 128),
                     mdesc(w2s + 256 * kk, 128, (kH / 8) * 128), idesc_bf16(kH), kk > 0 ? 1u : 0u);
        mma_commit(c.bar);
    }
    ok = __syncthreads_and(mbar_wait(c.bar, phase));
    phase ^= 1;
    if (!ok) return false;
    tc_after();
    hidden_epilogue(c.tmem_row, 0, bias + kH, a2, tid);
    // layer 3: D[:, 0:16) = H2 (128 x 64) * W3^T (rows 2..15 of W3 are zero)
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    if (tid == 0) {
#pragma unroll
        for (int kk = 0; kk < kH / 16; ++kk)
            mma_bf16(c.tmem, mdesc(a2s + 256 * kk, 128, (kH / 8) * 128), mdesc(w3s + 256 * kk, 128, (kH / 8) * 128),
                     idesc_bf16(kN3), kk > 0 ? 1u : 0u);
        mma_commit(c.bar);
    }
    ok = __syncthreads_and(mbar_wait(c.bar, phase));
    phase ^= 1;
    if (!ok) return false;
    tc_after();
    float o[16];
    tmem_ld16(c.tmem_row, o);
    if (pix < pv.npx) {
        const float y0 = o[0] + bias[2 * kH], y1 = o[1] + bias[2 * kH + 1];
        pv.ivl[pix] = has ? to_interval(pv.v, y0, y1) : make_int2(0, -1);
        if (pv.raw) pv.raw[pix] = make_float2(y0, y1);
    }
    tc_before();
    __syncthreads();
    tc_after();
    return true;
}

// The rays of an 8x4 pixel block start their intervals together: every usable
// interval of the block begins at the block's earliest start.  Evaluating more
// samples ahead of a proposed interval never loses a crossing (it can only
// find an earlier one), and the lanes of a march tile (8x4 pixels by default)
// then step through the same sample indices.  Warp per block.
constexpr int kIvlBlockW = 8, kIvlBlockH = 4;

__device__ __forceinline__ void ivl_block(int2* ivl, int W, int Hh, uint64_t blk, int lane) {
    const uint64_t bw = (uint64_t)((W + kIvlBlockW - 1) / kIvlBlockW);
    const int x = (int)(blk % bw) * kIvlBlockW + (lane % kIvlBlockW);
    const int y = (int)(blk / bw) * kIvlBlockH + (lane / kIvlBlockW);
    const bool in = x < W && y < Hh;
    int2 iv = make_int2(0, -1);
    if (in) iv = ivl[(uint64_t)y * (uint64_t)W + (uint64_t)x];
    const bool ok = in && iv.x >= 1 && iv.x < iv.y;
    const int m = __reduce_min_sync(0xffffffffu, ok ? iv.x : 0x7fffffff);
    if (ok && m < iv.x) ivl[(uint64_t)y * (uint64_t)W + (uint64_t)x] = make_int2(m, iv.y);
}

__global__ void k_ivl_blocks(int2* ivl, int W, int Hh, uint64_t nblk) {
    const uint64_t blk = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (blk >= nblk) return;  // warp-uniform
    ivl_block(ivl, W, Hh, blk, threadIdx.x & 31);
}

__global__ void k_ivl_blocks_b(const ProposeView* __restrict__ views, const uint64_t* __restrict__ pfx, int nviews,
                               uint64_t nblk) {
    const uint64_t blk = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    if (blk >= nblk) return;  // warp-uniform
    int lo = 0, hi = nviews - 1;  // the view of block blk: largest v with pfx[v] <= blk
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pfx[mid] <= blk) lo = mid;
        else hi = mid - 1;
    }
    const ProposeView& v = views[lo];
    ivl_block(v.ivl, v.f.W, v.f.Hh, blk - pfx[lo], threadIdx.x & 31);
}

uint64_t ivl_blocks(int W, int Hh) {
    return (uint64_t)((W + kIvlBlockW - 1) / kIvlBlockW) * (uint64_t)((Hh + kIvlBlockH - 1) / kIvlBlockH);
}

template <bool BATCH>
__global__ void __launch_bounds__(kRows) k_propose(const ProposeArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        const uint4* src = (const uint4*)a.weights;
        uint4* dst = (uint4*)(sm + kSmW1);
        for (uint32_t i = tid; i < kWeightBytes / 16; i += kRows) dst[i] = src[i];
        float* b = (float*)(sm + kSmBias);
        for (int i = tid; i < 2 * kH + kO; i += kRows) b[i] = a.bias[i];
    }
    ProposeCta c;
    c.sm = sm;
    c.sbase = smem_u32(sm);
    c.bar = c.sbase + kSmBar;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(c.bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(c.sbase + kSmTmem),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_before();
    __syncthreads();
    tc_after();
    c.tmem = *(volatile uint32_t*)(sm + kSmTmem);
    c.tmem_row = c.tmem + ((uint32_t)(warp * 32) << 16);  // this warp's 32 lanes
    uint32_t phase = 0;
    bool ok = true;
    for (uint64_t t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
        if (BATCH) {
            int lo = 0, hi = a.nviews - 1;  // the view of tile t: largest v with tile_pfx[v] <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.tile_pfx[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            ok = propose_tile(a.views[lo], t - a.tile_pfx[lo], c, phase);
        } else {
            ok = propose_tile(a.one, t, c, phase);
        }
    }
    const uint32_t tmem = c.tmem, bar = c.bar;
    if (!ok) {
        // an MMA did not complete in time: report, give the last commit another
        // bounded wait, then release the tensor memory
        if (tid == 0) atomicOr(a.status, 8u);
        mbar_wait(bar, phase ^ 1);
    }
    tc_before();
    __syncthreads();
    tc_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

// Diagnostics: the bounded wait of k_propose on an mbarrier that never
// completes (two arrivals expected, one made).  The wait gives up after
// `limit` polls, the kernel reports status bit 8 as k_propose does and exits.
__global__ void k_wait_selftest(unsigned int* status, uint32_t limit) {
    __shared__ __align__(8) uint64_t bar_mem;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&bar_mem);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(2u) : "memory");
        asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
    }
    __syncthreads();
    const bool ok = __syncthreads_and(mbar_wait(bar, 0, limit));
    if (!ok && threadIdx.x == 0) atomicOr(status, 8u);
}

// ---- training (FP32 SIMT) --------------------------------------------------------------

// Forward pass of a batch: z1, z2 (pre-activations), y; with targets also the
// pinball-loss gradient dy (scaled by 1/n) and the loss sum.
__global__ void __launch_bounds__(128) k_train_fwd(const float* __restrict__ P, const float* __restrict__ X,
                                                   const float* __restrict__ T, uint32_t n, float tau_lo,
                                                   float tau_hi, float* __restrict__ z1, float* __restrict__ z2,
                                                   float* __restrict__ y, float* __restrict__ dy,
                                                   float* __restrict__ loss) {
    __shared__ float w[kProposalParams];
    for (int i = threadIdx.x; i < kProposalParams; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (b < n) {
        float x[kF];
#pragma unroll
        for (int k = 0; k < kF; ++k) x[k] = X[(uint64_t)b * kF + k];
        float h1[kH];
        for (int j = 0; j < kH; ++j) {
            float s = w[oB1 + j];
#pragma unroll
            for (int k = 0; k < kF; ++k) s += w[oW1 + j * kF + k] * x[k];
            if (z1) z1[(uint64_t)b * kH + j] = s;
            h1[j] = gelu(s);
        }
        float yo[kO] = {w[oB3], w[oB3 + 1]};
        for (int j = 0; j < kH; ++j) {
            float s = w[oB2 + j];
#pragma unroll 8
            for (int k = 0; k < kH; ++k) s += w[oW2 + j * kH + k] * h1[k];
            if (z2) z2[(uint64_t)b * kH + j] = s;
            const float h = gelu(s);
            yo[0] += w[oW3 + j] * h;
            yo[1] += w[oW3 + kH + j] * h;
        }
        y[(uint64_t)b * kO] = yo[0];
        y[(uint64_t)b * kO + 1] = yo[1];
        if (T) {
            const float t = T[b], inv = 1.0f / (float)n;
            const float e0 = t - yo[0], e1 = t - yo[1];
            l = fmaxf(tau_lo * e0, (tau_lo - 1.0f) * e0) + fmaxf(tau_hi * e1, (tau_hi - 1.0f) * e1);
            dy[(uint64_t)b * kO] = (e0 > 0.0f ? -tau_lo : 1.0f - tau_lo) * inv;
            dy[(uint64_t)b * kO + 1] = (e1 > 0.0f ? -tau_hi : 1.0f - tau_hi) * inv;
        }
    }
    if (loss) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss, l);
    }
}

// Backward through the activations: dz2 = (dy W3) * gelu'(z2), dz1 = (dz2 W2) * gelu'(z1).
__global__ void __launch_bounds__(128) k_train_bwd(const float* __restrict__ P, uint32_t n,
                                                   const float* __restrict__ z1, const float* __restrict__ z2,
                                                   const float* __restrict__ dy, float* __restrict__ dz1,
                                                   float* __restrict__ dz2) {
    __shared__ float w[kProposalParams];
    for (int i = threadIdx.x; i < kProposalParams; i += blockDim.x) w[i] = P[i];
    __syncthreads();
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const float d0 = dy[(uint64_t)b * kO], d1 = dy[(uint64_t)b * kO + 1];
    float g2[kH];
    for (int k = 0; k < kH; ++k) {
        g2[k] = (d0 * w[oW3 + k] + d1 * w[oW3 + kH + k]) * gelu_grad(z2[(uint64_t)b * kH + k]);
        dz2[(uint64_t)b * kH + k] = g2[k];
    }
    for (int k = 0; k < kH; ++k) {
        float s = 0.0f;
#pragma unroll 8
        for (int j = 0; j < kH; ++j) s += g2[j] * w[oW2 + j * kH + k];
        dz1[(uint64_t)b * kH + k] = s * gelu_grad(z1[(uint64_t)b * kH + k]);
    }
}

// Parameter gradients: every thread owns parameters p = tid + 256 i and sums
// their per-sample terms over this block's chunk of the batch into the block's
// row of `partial`; k_grad_reduce adds the rows in block order, so a training
// step gives the same bits on every run (checkpoints resume exactly).
constexpr int kGradThreads = 256;
constexpr int kGradStage = 8;  // samples staged in shared memory at a time
constexpr int kRowFloats = kF + 4 * kH + kO;  // x, h1, h2, dz1, dz2, dy

__global__ void __launch_bounds__(kGradThreads) k_train_grad(const float* __restrict__ X, uint32_t n,
                                                             const float* __restrict__ z1,
                                                             const float* __restrict__ z2,
                                                             const float* __restrict__ dz1,
                                                             const float* __restrict__ dz2,
                                                             const float* __restrict__ dy, uint32_t chunk,
                                                             float* __restrict__ partial) {
    __shared__ float rows[kGradStage][kRowFloats];
    constexpr int kPer = (kProposalParams + kGradThreads - 1) / kGradThreads;
    float acc[kPer];
    int ia[kPer], ib[kPer];  // per owned parameter: offsets of its two factors in a staged row (-1: 1.0)
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        acc[i] = 0.0f;
        const int p = threadIdx.x + kGradThreads * i;
        ia[i] = ib[i] = -2;  // -2: not a parameter
        if (p < oB1) { ia[i] = kF + 2 * kH + p / kF; ib[i] = p % kF; }                         // dz1[j] x[k]
        else if (p < oW2) { ia[i] = kF + 2 * kH + (p - oB1); ib[i] = -1; }                     // dz1[j]
        else if (p < oB2) { ia[i] = kF + 3 * kH + (p - oW2) / kH; ib[i] = kF + (p - oW2) % kH; }  // dz2[j] h1[k]
        else if (p < oW3) { ia[i] = kF + 3 * kH + (p - oB2); ib[i] = -1; }                     // dz2[j]
        else if (p < oB3) { ia[i] = kF + 4 * kH + (p - oW3) / kH; ib[i] = kF + kH + (p - oW3) % kH; }  // dy[o] h2[k]
        else if (p < kProposalParams) { ia[i] = kF + 4 * kH + (p - oB3); ib[i] = -1; }          // dy[o]
    }
    const uint64_t b0 = (uint64_t)blockIdx.x * chunk;
    const uint64_t b1 = (b0 + chunk < (uint64_t)n) ? b0 + chunk : (uint64_t)n;
    for (uint64_t s0 = b0; s0 < b1; s0 += kGradStage) {
        const int m = (b1 - s0 < (uint64_t)kGradStage) ? (int)(b1 - s0) : kGradStage;
        __syncthreads();
        for (int e = threadIdx.x; e < m * kRowFloats; e += kGradThreads) {
            const int r = e / kRowFloats, c = e % kRowFloats;
            const uint64_t b = s0 + r;
            float v;
            if (c < kF) v = X[b * kF + c];
            else if (c < kF + kH) v = gelu(z1[b * kH + (c - kF)]);
            else if (c < kF + 2 * kH) v = gelu(z2[b * kH + (c - kF - kH)]);
            else if (c < kF + 3 * kH) v = dz1[b * kH + (c - kF - 2 * kH)];
            else if (c < kF + 4 * kH) v = dz2[b * kH + (c - kF - 3 * kH)];
            else v = dy[b * kO + (c - kF - 4 * kH)];
            rows[r][c] = v;
        }
        __syncthreads();
        for (int r = 0; r < m; ++r) {
#pragma unroll
            for (int i = 0; i < kPer; ++i) {
                if (ia[i] == -2) continue;
                const float fa = rows[r][ia[i]];
                acc[i] += (ib[i] < 0) ? fa : fa * rows[r][ib[i]];
            }
        }
    }
    float* row = partial + (uint64_t)blockIdx.x * kProposalParams;
#pragma unroll
    for (int i = 0; i < kPer; ++i)
        if (ia[i] != -2) row[threadIdx.x + kGradThreads * i] = acc[i];
}

__global__ void k_grad_reduce(const float* __restrict__ partial, uint32_t rows, float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kProposalParams) return;
    float s = 0.0f;
    for (uint32_t r = 0; r < rows; ++r) s += partial[(uint64_t)r * kProposalParams + p];
    grad[p] = s;
}

__global__ void k_adam(float* __restrict__ P, float* __restrict__ G, float* __restrict__ M, float* __restrict__ V,
                       float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kProposalParams) return;
    const float g = G[i];
    const float m = b1 * M[i] + (1.0f - b1) * g;
    const float v = b2 * V[i] + (1.0f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    G[i] = 0.0f;
}

// ---- judge ----------------------------------------------------------------------------

__global__ void k_judge(const float* __restrict__ dref, const float* __restrict__ dtest, uint64_t n, float tol,
                        unsigned long long* __restrict__ acc, unsigned int* __restrict__ maxerr) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    bool hr = false, ht = false, within = false;
    float err = 0.0f;
    if (i < n) {
        const float a = dref[i], b = dtest[i];
        hr = a > 0.0f;
        ht = b > 0.0f;
        if (hr && ht) {
            err = fabsf(b - a);
            within = err <= tol;
        }
    }
    const unsigned m_hr = __ballot_sync(0xffffffffu, hr), m_ht = __ballot_sync(0xffffffffu, ht);
    const unsigned m_mis = __ballot_sync(0xffffffffu, hr != ht), m_in = __ballot_sync(0xffffffffu, within);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err = fmaxf(err, __shfl_xor_sync(0xffffffffu, err, o));
    if ((threadIdx.x & 31) == 0) {
        if (m_hr) atomicAdd(acc + 0, (unsigned long long)__popc(m_hr));
        if (m_ht) atomicAdd(acc + 1, (unsigned long long)__popc(m_ht));
        if (m_mis) atomicAdd(acc + 2, (unsigned long long)__popc(m_mis));
        if (m_in) atomicAdd(acc + 3, (unsigned long long)__popc(m_in));
        if (err > 0.0f) atomicMax(maxerr, __float_as_uint(err));
    }
}

// Per-frame judge: the sample of a frame is every started pixel of the 8x4
// pixel blocks (one march tile each) whose hashed block index (lowbias32 of
// index ^ seed) is 0 modulo the stride, so the sampled rays march together.
__device__ __forceinline__ bool judge_sampled(uint64_t i, uint32_t width, uint32_t seed, uint32_t stride) {
    const uint32_t px = (uint32_t)(i % width), py = (uint32_t)(i / width);
    uint32_t x = ((py >> 2) * ((width + 7u) >> 3) + (px >> 3)) ^ seed;
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x % stride == 0u;
}

// Start plane of the sample: the learned march's start depth where sampled, 1 (no ray) elsewhere.
__global__ void k_judge_starts(const float* __restrict__ z, float* __restrict__ zs, uint64_t n, uint32_t width,
                               uint32_t seed, uint32_t stride) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < n) zs[i] = judge_sampled(i, width, seed, stride) ? z[i] : 1.0f;
}

// acc: frames, sampled, hits_ref, hits_test, mask_mismatch, within_tol, max |error| bits.
__global__ void k_judge_sample(const float* __restrict__ zs, const float* __restrict__ dref,
                               const float* __restrict__ dtest, uint64_t n, float tol,
                               unsigned long long* __restrict__ acc) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    bool s = false, hr = false, ht = false, within = false;
    float err = 0.0f;
    if (i < n && zs[i] != 1.0f) {
        s = true;
        const float a = dref[i], b = dtest[i];
        hr = a > 0.0f;
        ht = b > 0.0f;
        if (hr && ht) {
            err = fabsf(b - a);
            within = err <= tol;
        }
    }
    const unsigned m_s = __ballot_sync(0xffffffffu, s), m_hr = __ballot_sync(0xffffffffu, hr);
    const unsigned m_ht = __ballot_sync(0xffffffffu, ht), m_mis = __ballot_sync(0xffffffffu, hr != ht);
    const unsigned m_in = __ballot_sync(0xffffffffu, within);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) err = fmaxf(err, __shfl_xor_sync(0xffffffffu, err, o));
    if ((threadIdx.x & 31) == 0 && m_s) {
        atomicAdd(acc + 1, (unsigned long long)__popc(m_s));
        if (m_hr) atomicAdd(acc + 2, (unsigned long long)__popc(m_hr));
        if (m_ht) atomicAdd(acc + 3, (unsigned long long)__popc(m_ht));
        if (m_mis) atomicAdd(acc + 4, (unsigned long long)__popc(m_mis));
        if (m_in) atomicAdd(acc + 5, (unsigned long long)__popc(m_in));
        if (err > 0.0f) atomicMax(acc + 6, (unsigned long long)__float_as_uint(err));
    }
    if (i == 0) atomicAdd(acc + 0, 1ull);
}

// Host FP32 -> BF16, round to nearest even (NaN kept quiet).
uint16_t to_bf16(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}

}  // namespace

int ensure_occupancy(fm_ctx* ctx, fm_scene* s, cudaStream_t st) {
    if (s->occ_valid) return FM_OK;
    const size_t cells = (size_t)kOcc * kOcc * kOcc;
    if (!s->d_occ && cudaMalloc(&s->d_occ, cells * sizeof(uint16_t)) != cudaSuccess)
        return set_err(ctx, FM_ERR_OOM, "occupancy grid allocation failed");
    float vox[3];
    for (int k = 0; k < 3; ++k) vox[k] = (s->max[k] - s->min[k]) / (float)kOcc;
    k_occ_density<<<(unsigned)((cells + 127) / 128), 128, 0, st>>>(grid_dev(s), make_kernel(s->support), s->min[0],
                                                                   s->min[1], s->min[2], vox[0], vox[1], vox[2],
                                                                   (__half*)s->d_occ);
    FM_CUDA(ctx, cudaGetLastError());
    s->occ_valid = true;
    return FM_OK;
}

namespace {

FeatArgs make_feat(const fm_scene* s, const fm_camera* cam, const float* zbuf, const float* zlow) {
    FeatArgs f;
    const int W = cam->width, Hh = cam->height;
    for (int i = 0; i < 16; ++i) f.ipv[i] = cam->inv_proj_view[i];
    for (int k = 0; k < 3; ++k) f.cam[k] = cam->position[k];
    f.twoWinv = 2.0f / (float)W;
    f.twoHinv = 2.0f / (float)Hh;
    f.W = W;
    f.Hh = Hh;
    f.lw = (W + kLow - 1) / kLow;
    f.zbuf = zbuf;
    f.zlow = zlow;
    f.occ = (const __half*)s->d_occ;
    for (int k = 0; k < 3; ++k) {
        const float ext = s->max[k] - s->min[k];
        f.omin[k] = s->min[k];
        f.oinv[k] = (float)kOcc / ext;
        f.bmin[k] = s->min[k];
        f.binv[k] = 1.0f / ext;
    }
    f.H = s->support;
    f.invH = 1.0f / s->support;
    return f;
}

IvlArgs make_ivl(const fm_scene* s, const fm_march_params* p, const fm_proposal* pr) {
    IvlArgs v;
    v.H = s->support;
    v.step = p->step_size;
    v.max_steps = p->max_steps;
    v.margin_lo = pr->margin_lo;
    v.margin_hi = pr->margin_hi;
    v.min_near = pr->min_near;
    return v;
}

int feat_args(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const float* zbuf, cudaStream_t st,
              FeatArgs& f) {
    const int W = cam->width, Hh = cam->height;
    const int lw = (W + kLow - 1) / kLow, lh = (Hh + kLow - 1) / kLow;
    if (!grow_buf(ctx->prop_low, (size_t)lw * lh * sizeof(float)))
        return set_err(ctx, FM_ERR_OOM, "low-resolution depth allocation failed");
    k_lowres<<<(lw * lh + 255) / 256, 256, 0, st>>>(zbuf, W, Hh, lw, lh, (float*)ctx->prop_low.p);
    FM_CUDA(ctx, cudaGetLastError());
    f = make_feat(s, cam, zbuf, (const float*)ctx->prop_low.p);
    return FM_OK;
}

// Batched low-resolution depth: thread per low-resolution pixel of all views.
__global__ void k_lowres_b(const ProposeView* __restrict__ views, const uint64_t* __restrict__ low_pfx, int nviews,
                           uint64_t nlow) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nlow) return;
    int lo = 0, hi = nviews - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (low_pfx[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const FeatArgs& f = views[lo].f;
    const uint64_t l = t - low_pfx[lo];
    const int bx = (int)(l % (uint64_t)f.lw), by = (int)(l / (uint64_t)f.lw);
    float m = 1.0f;
    for (int y = by * kLow; y < min(by * kLow + kLow, f.Hh); ++y)
        for (int x = bx * kLow; x < min(bx * kLow + kLow, f.W); ++x) m = fminf(m, f.zbuf[(uint64_t)y * f.W + x]);
    const_cast<float*>(f.zlow)[l] = m;
}

}  // namespace

size_t propose_view_bytes() { return sizeof(ProposeView); }

uint64_t propose_low_pixels(const fm_camera* cam) {
    return (uint64_t)((cam->width + kLow - 1) / kLow) * (uint64_t)((cam->height + kLow - 1) / kLow);
}

void propose_view(const fm_scene* s, const fm_camera* cam, const fm_march_params* p, const float margins[3],
                  const float* zbuf, float* zlow, int2* ivl, void* out) {
    fm_proposal pr;
    pr.margin_lo = margins[0];
    pr.margin_hi = margins[1];
    pr.min_near = margins[2];
    ProposeView v;
    v.f = make_feat(s, cam, zbuf, zlow);
    v.v = make_ivl(s, p, &pr);
    v.ivl = ivl;
    v.raw = nullptr;
    v.npx = (uint64_t)cam->width * cam->height;
    std::memcpy(out, &v, sizeof(v));
}

int proposal_weights(fm_ctx* ctx, const fm_proposal* pr, DevBuf& w, DevBuf& b, float margins[3], cudaStream_t st) {
    margins[0] = pr->margin_lo;
    margins[1] = pr->margin_hi;
    margins[2] = pr->min_near;
    if (!grow_buf(w, kWeightBytes) || !grow_buf(b, (2 * kH + kO) * sizeof(float)))
        return set_err(ctx, FM_ERR_OOM, "proposal copy allocation failed");
    FM_CUDA(ctx, cudaMemcpyAsync(w.p, pr->d_weights, kWeightBytes, cudaMemcpyDeviceToDevice, st));
    FM_CUDA(ctx, cudaMemcpyAsync(b.p, pr->d_bias, (2 * kH + kO) * sizeof(float), cudaMemcpyDeviceToDevice, st));
    return FM_OK;
}

int launch_propose_batch(fm_ctx* ctx, const ProposeBatchDev& b, cudaStream_t st) {
    if (b.nlow)
        k_lowres_b<<<(unsigned)((b.nlow + 255) / 256), 256, 0, st>>>((const ProposeView*)b.views, b.low_pfx,
                                                                     b.nviews, b.nlow);
    ProposeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.views = (const ProposeView*)b.views;
    a.tile_pfx = b.tile_pfx;
    a.nviews = b.nviews;
    a.ntiles = b.ntiles;
    a.weights = (const uint8_t*)b.weights;
    a.bias = b.bias;
    a.status = ctx->d_status;
    FM_CUDA(ctx, cudaFuncSetAttribute(k_propose<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmRequest));
    uint64_t grid = (uint64_t)ctx->sm_count * kCtasPerSm;
    if (grid > b.ntiles) grid = b.ntiles;
    if (grid) k_propose<true><<<(unsigned)grid, kRows, kSmRequest, st>>>(a);
    if (b.nblk)
        k_ivl_blocks_b<<<(unsigned)((b.nblk * 32 + 255) / 256), 256, 0, st>>>((const ProposeView*)b.views, b.blk_pfx,
                                                                             b.nviews, b.nblk);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

uint64_t propose_view_blocks(const fm_camera* cam) { return ivl_blocks(cam->width, cam->height); }

int launch_features(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const float* zbuf, float* feat, float* t0,
                    cudaStream_t st) {
    int rc = ensure_occupancy(ctx, s, st);
    if (rc) return rc;
    FeatArgs f;
    if ((rc = feat_args(ctx, s, cam, zbuf, st, f)) != FM_OK) return rc;
    const uint64_t npx = (uint64_t)cam->width * cam->height;
    k_features<<<(unsigned)((npx + 127) / 128), 128, 0, st>>>(f, feat, t0);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

int launch_propose(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const fm_march_params* p, const fm_proposal* pr,
                   const float* zbuf, int2* ivl, float2* raw, cudaStream_t st) {
    int rc = ensure_occupancy(ctx, s, st);
    if (rc) return rc;
    ProposeArgs a;
    std::memset(&a, 0, sizeof(a));
    if ((rc = feat_args(ctx, s, cam, zbuf, st, a.one.f)) != FM_OK) return rc;
    a.one.v = make_ivl(s, p, pr);
    a.one.ivl = ivl;
    a.one.raw = raw;
    a.one.npx = (uint64_t)cam->width * cam->height;
    a.ntiles = (a.one.npx + kRows - 1) / kRows;
    a.weights = (const uint8_t*)pr->d_weights;
    a.bias = pr->d_bias;
    a.status = ctx->d_status;
    FM_CUDA(ctx, cudaFuncSetAttribute(k_propose<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmRequest));
    uint64_t grid = (uint64_t)ctx->sm_count * kCtasPerSm;
    if (grid > a.ntiles) grid = a.ntiles;
    k_propose<false><<<(unsigned)grid, kRows, kSmRequest, st>>>(a);
    const uint64_t nblk = ivl_blocks(cam->width, cam->height);
    k_ivl_blocks<<<(unsigned)((nblk * 32 + 255) / 256), 256, 0, st>>>(ivl, cam->width, cam->height, nblk);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

int judge_start(fm_ctx* ctx, fm_scene* s, const fm_camera* cam, const fm_march_params* p, const float* z,
                cudaStream_t st) {
    const uint64_t npx = (uint64_t)cam->width * cam->height;
    const bool fresh = ctx->judge_acc.p == nullptr;
    if (!grow_buf(ctx->judge_z, npx * 4) || !grow_buf(ctx->judge_ref, npx * 4) || !grow_buf(ctx->judge_acc, 64))
        return set_err(ctx, FM_ERR_OOM, "judge buffer allocation failed");
    if (fresh) FM_CUDA(ctx, cudaMemsetAsync(ctx->judge_acc.p, 0, 64, st));
    const uint32_t seed = (uint32_t)(ctx->judge_seq++ * 0x9E3779B9ull);
    float* zs = (float*)ctx->judge_z.p;
    k_judge_starts<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(z, zs, npx, (uint32_t)cam->width, seed,
                                                                   ctx->judge_stride);
    FM_CUDA(ctx, cudaGetLastError());
    // the plain march of the sample: same settings, its own start plane, hit
    // distances and long-ray queue
    fm_march_params q = *p;
    q.flags = FM_MARCH_EXTERNAL_DEPTH;
    MarchOutDev o{};
    o.start_depth = zs;
    o.depth = (float*)ctx->judge_ref.p;
    const int stats = ctx->stats_enabled;
    ctx->stats_enabled = 0;  // the counters describe the learned march
    const int rc = launch_march(ctx, s, cam, &q, o, st, &ctx->judge_longq);
    ctx->stats_enabled = stats;
    return rc;
}

int judge_finish(fm_ctx* ctx, const float* learned_depth, uint64_t npx, cudaStream_t st) {
    k_judge_sample<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>((const float*)ctx->judge_z.p,
                                                                   (const float*)ctx->judge_ref.p, learned_depth, npx,
                                                                   ctx->judge_tol,
                                                                   (unsigned long long*)ctx->judge_acc.p);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace fm

using namespace fm;

namespace {

// Seeded initial parameters: U(-sqrt(6 / fan_in), +sqrt(6 / fan_in)), biases 0.
void init_params(uint64_t seed, float* P) {
    uint64_t x = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    auto next = [&]() {
        x ^= x >> 12;
        x ^= x << 25;
        x ^= x >> 27;
        return (double)((x * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int i = 0; i < kProposalParams; ++i) P[i] = 0.0f;
    const int ranges[3][3] = {{oW1, kH * kF, kF}, {oW2, kH * kH, kH}, {oW3, kO * kH, kH}};
    for (const auto& r : ranges) {
        const double lim = std::sqrt(6.0 / (double)r[2]);
        for (int i = 0; i < r[1]; ++i) P[r[0] + i] = (float)((2.0 * next() - 1.0) * lim);
    }
}

}  // namespace

extern "C" {

int fm_proposal_create(fm_ctx* ctx, const float* params, float margin_lo, float margin_hi, float min_near,
                       fm_proposal** out) {
    if (!ctx) return FM_ERR_INVALID;
    if (!out || !params) return set_err(ctx, FM_ERR_INVALID, "parameters or output handle pointer are NULL");
    *out = nullptr;
    for (int i = 0; i < kProposalParams; ++i)
        if (!std::isfinite(params[i])) return set_err(ctx, FM_ERR_INVALID, "proposal parameters are not finite");
    if (!std::isfinite(margin_lo) || !std::isfinite(margin_hi) || margin_lo < 0.0f || margin_hi < 0.0f ||
        !std::isfinite(min_near) || min_near < 0.0f)
        return set_err(ctx, FM_ERR_INVALID, "margins and min_near must be finite and >= 0");
    std::vector<uint8_t> img(kWeightBytes, 0);
    auto put = [&](uint32_t base, int n, int K, int rows, const float* W) {
        for (int r = 0; r < rows; ++r)
            for (int k = 0; k < K; ++k) {
                const uint16_t v = r < n ? to_bf16(W[r * K + k]) : 0;
                std::memcpy(&img[base - kSmW1 + canon_off(r, k, K)], &v, 2);
            }
    };
    put(kSmW1, kH, kF, kH, params + oW1);
    put(kSmW2, kH, kH, kH, params + oW2);
    put(kSmW3, kO, kH, kN3, params + oW3);
    std::vector<float> bias(2 * kH + kO);
    for (int j = 0; j < kH; ++j) bias[j] = params[oB1 + j];
    for (int j = 0; j < kH; ++j) bias[kH + j] = params[oB2 + j];
    bias[2 * kH] = params[oB3];
    bias[2 * kH + 1] = params[oB3 + 1];
    cudaSetDevice(ctx->device);
    fm_proposal* p = new (std::nothrow) fm_proposal();
    if (!p) return set_err(ctx, FM_ERR_OOM, "host allocation failed");
    p->ctx = ctx;
    p->margin_lo = margin_lo;
    p->margin_hi = margin_hi;
    p->min_near = min_near;
    if (cudaMalloc(&p->d_weights, kWeightBytes) != cudaSuccess ||
        cudaMalloc(&p->d_bias, bias.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(p->d_weights, img.data(), kWeightBytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(p->d_bias, bias.data(), bias.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(p->d_weights);
        cudaFree(p->d_bias);
        delete p;
        return set_err(ctx, FM_ERR_OOM, "proposal upload failed");
    }
    *out = p;
    return FM_OK;
}

void fm_proposal_destroy(fm_proposal* p) {
    if (!p) return;
    fm_ctx* ctx = p->ctx;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();  // a launch on any stream may still read the weights
    if (ctx->proposal == p) ctx->proposal = nullptr;
    cudaFree(p->d_weights);
    cudaFree(p->d_bias);
    delete p;
}

int fm_set_proposal(fm_ctx* ctx, fm_proposal* p) {
    if (!ctx) return FM_ERR_INVALID;
    if (p && p->ctx != ctx) return set_err(ctx, FM_ERR_INVALID, "proposal belongs to another context");
    ctx->proposal = p;
    return FM_OK;
}

int fm_proposal_features(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const float* start_depth,
                         float* features, float* t0, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!s || !cam || !start_depth || !features) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    int rc = check_camera(ctx, cam, false);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_features(ctx, const_cast<fm_scene*>(s), cam, start_depth, features, t0, st);
}

int fm_proposal_intervals(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* params,
                          const float* start_depth, int32_t* intervals, float* near_far, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!s || !cam || !params || !start_depth || !intervals) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    if (!ctx->proposal) return set_err(ctx, FM_ERR_INVALID, "no proposal set (fm_set_proposal)");
    int rc = check_camera(ctx, cam, false);
    if (!rc) rc = check_params(ctx, params);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return launch_propose(ctx, const_cast<fm_scene*>(s), cam, params, ctx->proposal, start_depth, (int2*)intervals,
                          (float2*)near_far, st);
}

int fm_judge(fm_ctx* ctx, const float* depth_ref, const float* depth_test, uint64_t n, float tol,
             fm_judge_result* out, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!depth_ref || !depth_test || !out) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    if (!(tol >= 0.0f)) return set_err(ctx, FM_ERR_INVALID, "tolerance must be >= 0");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (!grow_buf(ctx->prop_judge, 64)) return set_err(ctx, FM_ERR_OOM, "judge buffer allocation failed");
    unsigned long long* acc = (unsigned long long*)ctx->prop_judge.p;
    unsigned int* mx = (unsigned int*)(acc + 4);
    FM_CUDA(ctx, cudaMemsetAsync(acc, 0, 64, st));
    if (n) k_judge<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(depth_ref, depth_test, n, tol, acc, mx);
    FM_CUDA(ctx, cudaGetLastError());
    unsigned long long h[5];
    FM_CUDA(ctx, cudaMemcpyAsync(h, acc, 40, cudaMemcpyDeviceToHost, st));
    FM_CUDA(ctx, cudaStreamSynchronize(st));
    fm_judge_result r{};
    r.pixels = n;
    r.hits_ref = h[0];
    r.hits_test = h[1];
    r.mask_mismatch = h[2];
    r.within_tol = h[3];
    const unsigned int mb = (unsigned int)(h[4] & 0xffffffffu);
    std::memcpy(&r.max_err, &mb, 4);
    r.tol = tol;
    *out = r;
    return FM_OK;
}

int fm_set_judge(fm_ctx* ctx, uint32_t stride, float tol) {
    if (!ctx) return FM_ERR_INVALID;
    if (!(tol >= 0.0f) || !std::isfinite(tol)) return set_err(ctx, FM_ERR_INVALID, "tolerance must be finite and >= 0");
    ctx->judge_stride = stride;
    ctx->judge_tol = tol;
    return FM_OK;
}

int fm_judge_frames(fm_ctx* ctx, fm_frame_judge* out, int reset) {
    if (!ctx) return FM_ERR_INVALID;
    if (!out) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    cudaSetDevice(ctx->device);
    fm_frame_judge r{};
    r.tol = ctx->judge_tol;
    if (ctx->judge_acc.p) {
        unsigned long long h[7];
        FM_CUDA(ctx, cudaDeviceSynchronize());  // judged marches may run on any stream
        FM_CUDA(ctx, cudaMemcpy(h, ctx->judge_acc.p, sizeof(h), cudaMemcpyDeviceToHost));
        r.frames = h[0];
        r.sampled = h[1];
        r.hits_ref = h[2];
        r.hits_test = h[3];
        r.mask_mismatch = h[4];
        r.within_tol = h[5];
        const unsigned int mb = (unsigned int)(h[6] & 0xffffffffu);
        std::memcpy(&r.max_err, &mb, 4);
        if (reset) FM_CUDA(ctx, cudaMemset(ctx->judge_acc.p, 0, 64));
    }
    *out = r;
    return FM_OK;
}

int fm_trainer_create(fm_ctx* ctx, uint64_t seed, const float* init, fm_trainer** out) {
    if (!ctx) return FM_ERR_INVALID;
    if (!out) return set_err(ctx, FM_ERR_INVALID, "output handle pointer is NULL");
    *out = nullptr;
    std::vector<float> P(kProposalParams);
    if (init) {
        for (int i = 0; i < kProposalParams; ++i) {
            if (!std::isfinite(init[i])) return set_err(ctx, FM_ERR_INVALID, "initial parameters are not finite");
            P[i] = init[i];
        }
    } else {
        init_params(seed, P.data());
    }
    cudaSetDevice(ctx->device);
    fm_trainer* t = new (std::nothrow) fm_trainer();
    if (!t) return set_err(ctx, FM_ERR_OOM, "host allocation failed");
    t->ctx = ctx;
    if (cudaMalloc(&t->d_p, 4 * kProposalParams * sizeof(float)) != cudaSuccess) {
        delete t;
        return set_err(ctx, FM_ERR_OOM, "trainer allocation failed");
    }
    cudaMemset(t->d_p, 0, 4 * kProposalParams * sizeof(float));
    cudaMemcpy(t->d_p, P.data(), kProposalParams * sizeof(float), cudaMemcpyHostToDevice);
    *out = t;
    return FM_OK;
}

void fm_trainer_destroy(fm_trainer* t) {
    if (!t) return;
    cudaSetDevice(t->ctx->device);
    cudaStreamSynchronize(t->ctx->stream);
    cudaFree(t->d_p);
    cudaFree(t->work.p);
    delete t;
}

int fm_trainer_step(fm_trainer* t, const float* features, const float* targets, uint32_t n, float lr, float tau_lo,
                    float tau_hi, float* loss) {
    if (!t) return FM_ERR_INVALID;
    fm_ctx* ctx = t->ctx;
    if (!features || !targets || n == 0) return set_err(ctx, FM_ERR_INVALID, "empty batch");
    if (!(lr > 0.0f) || !(tau_lo > 0.0f && tau_lo < 1.0f) || !(tau_hi > 0.0f && tau_hi < 1.0f))
        return set_err(ctx, FM_ERR_INVALID, "learning rate or quantiles out of range");
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    const size_t per = 4 * kH + 2 * kO;  // z1, z2, dz1, dz2, y, dy
    const uint32_t chunk = 64;
    const uint32_t gblocks = (n + chunk - 1) / chunk;
    if (n > t->cap) {
        FM_CUDA(ctx, cudaStreamSynchronize(st));
        const size_t bytes = (size_t)n * per * sizeof(float) + 64 + (size_t)gblocks * kProposalParams * sizeof(float);
        if (!grow_buf(t->work, bytes)) return set_err(ctx, FM_ERR_OOM, "trainer buffers");
        t->cap = n;
    }
    float* z1 = (float*)t->work.p;
    float* z2 = z1 + (size_t)n * kH;
    float* dz1 = z2 + (size_t)n * kH;
    float* dz2 = dz1 + (size_t)n * kH;
    float* y = dz2 + (size_t)n * kH;
    float* dy = y + (size_t)n * kO;
    float* lsum = dy + (size_t)n * kO;
    float* partial = lsum + 16;  // 64-byte aligned: the work buffer is, and n * per is a multiple of 4
    float* P = t->d_p;
    float* G = P + kProposalParams;
    float* M = G + kProposalParams;
    float* V = M + kProposalParams;
    FM_CUDA(ctx, cudaMemsetAsync(lsum, 0, sizeof(float), st));
    const unsigned blocks = (n + 127) / 128;
    k_train_fwd<<<blocks, 128, 0, st>>>(P, features, targets, n, tau_lo, tau_hi, z1, z2, y, dy, lsum);
    k_train_bwd<<<blocks, 128, 0, st>>>(P, n, z1, z2, dy, dz1, dz2);
    k_train_grad<<<gblocks, kGradThreads, 0, st>>>(features, n, z1, z2, dz1, dz2, dy, chunk, partial);
    k_grad_reduce<<<(kProposalParams + 255) / 256, 256, 0, st>>>(partial, gblocks, G);
    t->steps++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - (float)std::pow((double)b1, t->steps), c2 = 1.0f - (float)std::pow((double)b2, t->steps);
    k_adam<<<(kProposalParams + 255) / 256, 256, 0, st>>>(P, G, M, V, lr, b1, b2, 1e-8f, c1, c2);
    FM_CUDA(ctx, cudaGetLastError());
    if (loss) {
        float h = 0.0f;
        FM_CUDA(ctx, cudaMemcpyAsync(&h, lsum, sizeof(float), cudaMemcpyDeviceToHost, st));
        FM_CUDA(ctx, cudaStreamSynchronize(st));
        *loss = h / (float)n;
    }
    return FM_OK;
}

int fm_trainer_predict(fm_trainer* t, const float* features, uint32_t n, float* out) {
    if (!t) return FM_ERR_INVALID;
    fm_ctx* ctx = t->ctx;
    if (!features || !out) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    if (n == 0) return FM_OK;
    cudaSetDevice(ctx->device);
    k_train_fwd<<<(n + 127) / 128, 128, 0, ctx->stream>>>(t->d_p, features, nullptr, n, 0.5f, 0.5f, nullptr, nullptr,
                                                          out, nullptr, nullptr);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

int fm_selftest_wait_timeout(fm_ctx* ctx, uint32_t polls) {
    if (!ctx) return FM_ERR_INVALID;
    if (polls == 0 || polls > kWaitLimit) return set_err(ctx, FM_ERR_INVALID, "polls must be in [1, 2^22]");
    cudaSetDevice(ctx->device);
    k_wait_selftest<<<1, 128, 0, ctx->stream>>>(ctx->d_status, polls);
    FM_CUDA(ctx, cudaGetLastError());
    unsigned int* hs = (unsigned int*)ctx->h_pinned_small;
    FM_CUDA(ctx, cudaMemcpyAsync(hs, ctx->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost, ctx->stream));
    FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned int code = hs[0];
    if (code != 0) {
        FM_CUDA(ctx, cudaMemset(ctx->d_status, 0, sizeof(unsigned int)));
        return set_err(ctx, FM_ERR_DEVICE, "wait timed out: kernel status word " + std::to_string(code));
    }
    return FM_OK;
}

int fm_trainer_get_state(fm_trainer* t, float* host_state, int64_t* step) {
    if (!t) return FM_ERR_INVALID;
    if (!host_state || !step) return set_err(t->ctx, FM_ERR_INVALID, "NULL argument");
    cudaSetDevice(t->ctx->device);
    FM_CUDA(t->ctx, cudaStreamSynchronize(t->ctx->stream));
    const float* P = t->d_p;
    FM_CUDA(t->ctx, cudaMemcpy(host_state, P, kProposalParams * sizeof(float), cudaMemcpyDeviceToHost));
    FM_CUDA(t->ctx, cudaMemcpy(host_state + kProposalParams, P + 2 * kProposalParams,
                               2 * kProposalParams * sizeof(float), cudaMemcpyDeviceToHost));
    *step = t->steps;
    return FM_OK;
}

int fm_trainer_set_state(fm_trainer* t, const float* host_state, int64_t step) {
    if (!t) return FM_ERR_INVALID;
    if (!host_state) return set_err(t->ctx, FM_ERR_INVALID, "NULL argument");
    if (step < 0 || step > (int64_t)1 << 30) return set_err(t->ctx, FM_ERR_INVALID, "step out of range");
    for (int i = 0; i < 3 * kProposalParams; ++i)
        if (!std::isfinite(host_state[i]) || (i >= 2 * kProposalParams && host_state[i] < 0.0f))
            return set_err(t->ctx, FM_ERR_INVALID, "state is not finite (or a second moment is negative)");
    cudaSetDevice(t->ctx->device);
    FM_CUDA(t->ctx, cudaStreamSynchronize(t->ctx->stream));
    float* P = t->d_p;
    FM_CUDA(t->ctx, cudaMemcpy(P, host_state, kProposalParams * sizeof(float), cudaMemcpyHostToDevice));
    FM_CUDA(t->ctx, cudaMemset(P + kProposalParams, 0, kProposalParams * sizeof(float)));
    FM_CUDA(t->ctx, cudaMemcpy(P + 2 * kProposalParams, host_state + kProposalParams,
                               2 * kProposalParams * sizeof(float), cudaMemcpyHostToDevice));
    t->steps = (int)step;
    return FM_OK;
}

int fm_trainer_params(fm_trainer* t, float* host_params) {
    if (!t) return FM_ERR_INVALID;
    if (!host_params) return set_err(t->ctx, FM_ERR_INVALID, "NULL argument");
    cudaSetDevice(t->ctx->device);
    FM_CUDA(t->ctx, cudaStreamSynchronize(t->ctx->stream));
    FM_CUDA(t->ctx, cudaMemcpy(host_params, t->d_p, kProposalParams * sizeof(float), cudaMemcpyDeviceToHost));
    return FM_OK;
}

}  // extern "C"
