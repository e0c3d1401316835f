// march.cu -- per-pixel SPH iso-surface march on the GPU.
//
// Restates RayMarcher::PerPixel_Isotropic (src/app/AdvancedRenderer/
// RayMarcher.cpp:256-344) for every pixel at once:
//   ray setup      clip = (x * 2/W - 1, y * 2/H - 1, z_splat) at the pixel
//                  corner, world = InvProjectionView * clip / w,
//                  step = StepSize * normalize(world - camera)  (:268-274)
//   march          p += step; rho = sum_j W(x_j - p) over the 27 cells around
//                  p; hit at the first sample with rho >= iso      (:276-343)
//   skip           FM_SKIP_REFERENCE: the reference's flag/jump loop
//                  (:281-306, intersectAABB :51-62);  FM_SKIP_EXACT: samples in
//                  cells whose density upper bound is below iso are stepped
//                  over without evaluating, so results equal skip-off exactly
//   refinement     bisection between the last outside and first inside sample
//   normal         normalize(sum_j gradW(x_j - p_hit)) (:332-338, Kernel.cpp:34-52)
//   shading        composition.frag:132-184 fused into the epilogue
// Summation order is the canonical order: cells in increasing linear index,
// particles in cell-sorted order; every cell row (x-1..x+1 at fixed y, z) is
// one contiguous range of the sorted float4 array.  With --fmad=false every
// FP32 operation rounds like the reference's, so a pixel's result is
// bit-identical to the CPU restatement.
//
// Launch shape: 128-thread blocks covering 16x8 pixels; each warp owns an 8x4
// pixel tile, so the 32 rays of a warp sample neighbouring points and read the
// same cell rows (their loads coalesce or broadcast in L1).

#include <cuda_runtime.h>

#include "fm_internal.cuh"

namespace fm {
namespace {

struct MarchArgs {
    GridDev g;
    KernelDev k;
    float iso, step;
    int max_steps, bisect, skip_mode;
    float ipv[16];
    float cam[3];
    float cdir[3];
    int W, Hh;
    float twoWinv, twoHinv;
    const float* __restrict__ zbuf;
    float4* pos;
    float4* nrm;
    float* depth;
    float4* col;
    unsigned long long* stats;
    unsigned int* status;
};

constexpr int kTileW = 16, kTileH = 8, kThreads = 128;

struct Acc {
    uint32_t evals = 0;
    uint64_t cand = 0;
    uint32_t skipped = 0;
};

// Density at p whose cell is (cx, cy, cz); canonical order.
template <bool STATS>
__device__ __forceinline__ float density_cell(const GridDev& g, const KernelDev& k, int cx, int cy, int cz,
                                              float px, float py, float pz, Acc& acc) {
    if (STATS) acc.evals++;
    float rho = 0.0f;
    const int x0 = max(cx - 1, 0), x1 = min(cx + 1, g.dims[0] - 1);
    if (x0 > x1) return rho;
    const int z0 = max(cz - 1, 0), z1 = min(cz + 1, g.dims[2] - 1);
    const int y0 = max(cy - 1, 0), y1 = min(cy + 1, g.dims[1] - 1);
    for (int z = z0; z <= z1; ++z) {
        for (int y = y0; y <= y1; ++y) {
            const uint32_t row = ((uint32_t)z * (uint32_t)g.dims[1] + (uint32_t)y) * (uint32_t)g.dims[0];
            const uint32_t b = __ldg(g.start + row + x0), e = __ldg(g.start + row + x1 + 1);
            if (STATS) acc.cand += e - b;
            for (uint32_t j = b; j < e; ++j) {
                const float4 q = __ldg(g.pts + j);
                const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
                const float q2 = dot3(rx, ry, rz, rx, ry, rz);
                if (q2 < k.h2) rho = rho + w_in(k, q2);
            }
        }
    }
    return rho;
}

template <bool STATS>
__device__ __forceinline__ float density(const GridDev& g, const KernelDev& k, float px, float py, float pz,
                                         Acc& acc) {
    int cx, cy, cz;
    if (!sample_cell(g, px, py, pz, cx, cy, cz)) {
        if (STATS) acc.evals++;
        return 0.0f;
    }
    return density_cell<STATS>(g, k, cx, cy, cz, px, py, pz, acc);
}

__device__ __forceinline__ void grad_sum(const GridDev& g, const KernelDev& k, float px, float py, float pz, float& gx, float& gy,
                         float& gz) {
    gx = gy = gz = 0.0f;
    int cx, cy, cz;
    if (!sample_cell(g, px, py, pz, cx, cy, cz)) return;
    const int x0 = max(cx - 1, 0), x1 = min(cx + 1, g.dims[0] - 1);
    if (x0 > x1) return;
    for (int z = max(cz - 1, 0); z <= min(cz + 1, g.dims[2] - 1); ++z)
        for (int y = max(cy - 1, 0); y <= min(cy + 1, g.dims[1] - 1); ++y) {
            const uint32_t row = ((uint32_t)z * (uint32_t)g.dims[1] + (uint32_t)y) * (uint32_t)g.dims[0];
            const uint32_t b = __ldg(g.start + row + x0), e = __ldg(g.start + row + x1 + 1);
            for (uint32_t j = b; j < e; ++j) {
                const float4 q = __ldg(g.pts + j);
                const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
                const float q2 = dot3(rx, ry, rz, rx, ry, rz);
                if (q2 < k.h2 && q2 > 0.0f) gradw_acc(k, rx, ry, rz, q2, gx, gy, gz);
            }
        }
}

// glm min/max semantics (func_common.inl): min(x,y) = y<x ? y : x, max(x,y) = x<y ? y : x
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }

// The reference's empty-space skip loop (RayMarcher.cpp:284-306), capped.
__device__ __forceinline__ void ref_skip(const GridDev& g, float& px, float& py, float& pz, float sx, float sy, float sz,
                         unsigned int* status) {
    for (int it = 0; it < (1 << 20); ++it) {
        float fx = floorf((px - g.min[0]) * g.inv);
        float fy = floorf((py - g.min[1]) * g.inv);
        float fz = floorf((pz - g.min[2]) * g.inv);
        if (!(fx >= 0.0f && fx < (float)g.dims[0] && fy >= 0.0f && fy < (float)g.dims[1] && fz >= 0.0f &&
              fz < (float)g.dims[2]))
            return;
        int x = (int)fx, y = (int)fy, z = (int)fz;
        uint32_t c = (uint32_t)x + (uint32_t)y * (uint32_t)g.dims[0] + (uint32_t)z * (uint32_t)g.dims[0] * (uint32_t)g.dims[1];
        if (g.flag[c]) return;
        float b0x = g.min[0] + (float)x * g.cell, b0y = g.min[1] + (float)y * g.cell, b0z = g.min[2] + (float)z * g.cell;
        float b1x = b0x + g.cell, b1y = b0y + g.cell, b1z = b0z + g.cell;
        float tminx = (b0x - px) / sx, tminy = (b0y - py) / sy, tminz = (b0z - pz) / sz;
        float tmaxx = (b1x - px) / sx, tmaxy = (b1y - py) / sy, tmaxz = (b1z - pz) / sz;
        float t1x = gmin(tminx, tmaxx), t1y = gmin(tminy, tmaxy), t1z = gmin(tminz, tmaxz);
        float t2x = gmax(tminx, tmaxx), t2y = gmax(tminy, tmaxy), t2z = gmax(tminz, tmaxz);
        float tnear = gmax(gmax(t1x, t1y), t1z);
        float tfar = gmin(gmin(t2x, t2y), t2z);
        float t = (tnear < tfar) ? tfar : tnear;
        if (t >= 0.0f) {
            px = px + sx * t;
            py = py + sy * t;
            pz = pz + sz * t;
        }
        px = px + sx;
        py = py + sy;
        pz = pz + sz;
    }
    atomicOr(status, 1u);
}

// composition.frag:99-108
__device__ __forceinline__ float4 sample_floor(float ax, float ay, float az, float rx, float ry, float rz) {
    float s = -1.0f - ay;
    float tx = (rx * s) / ry, tz = (rz * s) / ry;
    float bx = ax + tx, bz = az + tz;
    (void)ry;
    float mx = bx - 2.0f * floorf(bx / 2.0f);
    float mz = bz - 2.0f * floorf(bz / 2.0f);
    float fx = (1.0f < mx) ? 0.0f : 1.0f;
    float fz = (1.0f < mz) ? 0.0f : 1.0f;
    float c = 0.25f + (fx + fz) / 4.0f;
    return make_float4(c, c, c, 0.5f);
}

// composition.frag:132-184, active branch.
__device__ __forceinline__ float4 shade(const MarchArgs& a, int px, int py, bool hit, float hx, float hy, float hz, float nx, float ny,
                        float nz) {
    float u = ((float)px + 0.5f) / (float)a.W;
    float v = ((float)py + 0.5f) / (float)a.Hh;
    float in0 = 2.0f * u - 1.0f, in1 = 2.0f * v - 1.0f;
    float o[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float add0 = a.ipv[0 * 4 + r] * in0 + a.ipv[1 * 4 + r] * in1;
        float add1 = a.ipv[2 * 4 + r] * 1.0f + a.ipv[3 * 4 + r] * 1.0f;
        o[r] = add0 + add1;
    }
    float vx = o[0] / o[3], vy = o[1] / o[3], vz = o[2] / o[3];
    if (!hit) {
        float4 f = sample_floor(a.cam[0], a.cam[1], a.cam[2], vx, vy, vz);
        return make_float4(0.75f * f.x, 0.75f * f.y, 0.75f * f.z, 0.75f * f.w);
    }
    float inv = 1.0f / sqrtf(dot3(vx, vy, vz, vx, vy, vz));
    float ix = vx * inv, iy = vy * inv, iz = vz * inv;
    const float eta = 1.333f;
    float dv = dot3(nx, ny, nz, ix, iy, iz);
    float kk = 1.0f - (eta * eta) * (1.0f - dv * dv);
    float rx = 0.0f, ry = 0.0f, rz = 0.0f;
    if (kk >= 0.0f) {
        float c = eta * dv + sqrtf(kk);
        rx = eta * ix - c * nx;
        ry = eta * iy - c * ny;
        rz = eta * iz - c * nz;
    }
    float4 fl = sample_floor(hx, hy, hz, rx, ry, rz);
    float f = -dot3(a.cdir[0], a.cdir[1], a.cdir[2], nx, ny, nz);
    float kd = (0.15f + 1.0f) - f * f;
    return make_float4(f * fl.x + kd * (120.0f / 255.0f), f * fl.y + kd * (185.0f / 255.0f),
                       f * fl.z + kd * (255.0f / 255.0f), f * fl.w + kd * (255.0f / 255.0f));
}

template <bool STATS>
__global__ void __launch_bounds__(kThreads) k_march(const MarchArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = blockIdx.x * kTileW + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * kTileH + (warp >> 1) * 4 + (lane >> 3);
    const bool valid = px < a.W && py < a.Hh;
    Acc acc;
    bool hit = false, started = false;
    float hx = 0.f, hy = 0.f, hz = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
    const uint64_t idx = (uint64_t)py * a.W + px;
    if (valid) {
        const float z = a.zbuf[idx];
        if (z != 1.0f) {
            started = true;
            const float cxp = (float)px * a.twoWinv - 1.0f;
            const float cyp = (float)py * a.twoHinv - 1.0f;
            float wh[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float add0 = a.ipv[0 * 4 + r] * cxp + a.ipv[1 * 4 + r] * cyp;
                float add1 = a.ipv[2 * 4 + r] * z + a.ipv[3 * 4 + r] * 1.0f;
                wh[r] = add0 + add1;
            }
            float p0 = wh[0] / wh[3], p1 = wh[1] / wh[3], p2 = wh[2] / wh[3];
            float dx = p0 - a.cam[0], dy = p1 - a.cam[1], dz = p2 - a.cam[2];
            float inv = 1.0f / sqrtf(dot3(dx, dy, dz, dx, dy, dz));
            const float sx = a.step * (dx * inv), sy = a.step * (dy * inv), sz = a.step * (dz * inv);
            float q0 = p0, q1 = p1, q2 = p2;  // previous sample
            for (int i = 0; i < a.max_steps; ++i) {
                p0 = p0 + sx;
                p1 = p1 + sy;
                p2 = p2 + sz;
                if (a.skip_mode == FM_SKIP_REFERENCE) ref_skip(a.g, p0, p1, p2, sx, sy, sz, a.status);
                int cx, cy, cz;
                float rho;
                if (!sample_cell(a.g, p0, p1, p2, cx, cy, cz)) {
                    if (outside_forever(a.g, p0, p1, p2, sx, sy, sz)) break;
                    if (STATS) acc.evals++;
                    rho = 0.0f;
                } else {
                    if (a.skip_mode == FM_SKIP_EXACT && cx >= 0 && cy >= 0 && cz >= 0 && cx < a.g.dims[0] &&
                        cy < a.g.dims[1] && cz < a.g.dims[2]) {
                        const uint32_t c = (uint32_t)cx + (uint32_t)cy * (uint32_t)a.g.dims[0] +
                                           (uint32_t)cz * (uint32_t)a.g.dims[0] * (uint32_t)a.g.dims[1];
                        if (__ldg(a.g.bound + c) < a.iso) {
                            if (STATS) acc.skipped++;
                            q0 = p0; q1 = p1; q2 = p2;
                            continue;
                        }
                    }
                    rho = density_cell<STATS>(a.g, a.k, cx, cy, cz, p0, p1, p2, acc);
                }
                if (rho >= a.iso) {
                    hit = true;
                    break;
                }
                q0 = p0; q1 = p1; q2 = p2;
            }
            if (hit) {
                float l0 = q0, l1 = q1, l2 = q2;
                for (int b = 0; b < a.bisect; ++b) {
                    float m0 = (l0 + p0) * 0.5f, m1 = (l1 + p1) * 0.5f, m2 = (l2 + p2) * 0.5f;
                    float rho = density<STATS>(a.g, a.k, m0, m1, m2, acc);
                    if (rho >= a.iso) { p0 = m0; p1 = m1; p2 = m2; }
                    else { l0 = m0; l1 = m1; l2 = m2; }
                }
                hx = p0; hy = p1; hz = p2;
                float gx, gy, gz;
                grad_sum(a.g, a.k, hx, hy, hz, gx, gy, gz);
                if (STATS) acc.evals++;
                float gi = 1.0f / sqrtf(dot3(gx, gy, gz, gx, gy, gz));
                nx = gx * gi; ny = gy * gi; nz = gz * gi;
            }
        }
        if (a.pos) a.pos[idx] = hit ? make_float4(hx, hy, hz, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.nrm) a.nrm[idx] = hit ? make_float4(nx, ny, nz, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.depth) {
            float d = 0.0f;
            if (hit) {
                float rx = hx - a.cam[0], ry = hy - a.cam[1], rz = hz - a.cam[2];
                d = sqrtf(dot3(rx, ry, rz, rx, ry, rz));
            }
            a.depth[idx] = d;
        }
        if (a.col) a.col[idx] = shade(a, px, py, hit, hx, hy, hz, nx, ny, nz);
    }
    if (STATS) {
        unsigned long long v[6] = {valid ? 1ull : 0ull, started ? 1ull : 0ull, hit ? 1ull : 0ull,
                                   (unsigned long long)acc.evals, (unsigned long long)acc.cand,
                                   (unsigned long long)acc.skipped};
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            unsigned long long x = v[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0 && x) atomicAdd(a.stats + j, x);
        }
    }
}

}  // namespace

int launch_march(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p,
                 const MarchOutDev& o, cudaStream_t st) {
    MarchArgs a;
    a.g = grid_dev(s);
    a.k = make_kernel(s->support);
    a.iso = p->iso_density;
    a.step = p->step_size;
    a.max_steps = p->max_steps;
    a.bisect = p->bisect_iters;
    a.skip_mode = p->skip_mode;
    for (int i = 0; i < 16; ++i) a.ipv[i] = cam->inv_proj_view[i];
    for (int i = 0; i < 3; ++i) a.cam[i] = cam->position[i];
    a.cdir[0] = cam->view[2];
    a.cdir[1] = cam->view[6];
    a.cdir[2] = cam->view[10];
    a.W = cam->width;
    a.Hh = cam->height;
    a.twoWinv = 2.0f / (float)cam->width;
    a.twoHinv = 2.0f / (float)cam->height;
    a.zbuf = o.start_depth;
    a.pos = o.pos;
    a.nrm = o.nrm;
    a.depth = o.depth;
    a.col = o.col;
    a.stats = ctx->stats_enabled ? ctx->d_stats : nullptr;
    a.status = ctx->d_status;
    dim3 grid((cam->width + kTileW - 1) / kTileW, (cam->height + kTileH - 1) / kTileH);
    if (a.stats) k_march<true><<<grid, kThreads, 0, st>>>(a);
    else k_march<false><<<grid, kThreads, 0, st>>>(a);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace fm
