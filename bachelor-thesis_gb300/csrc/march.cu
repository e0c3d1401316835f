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
//                  sub-cells whose density upper bound is below iso are stepped
//                  over without evaluating, so results equal skip-off exactly
//   refinement     bisection between the last outside and first inside sample
//   normal         normalize(sum_j gradW(x_j - p_hit)) (:332-338, Kernel.cpp:34-52)
//   shading        composition.frag:132-184 fused into the epilogue
//
// Summation order is the canonical order: the particles of the 27 cells in
// sorted order (cell, 2x2x2 sub-cell, input index).  Sub-cells whose box is
// out of reach of the sample (distance >= support radius, with a margin for
// rounding) hold only particles with W = 0 and are skipped; every other
// particle is added in order.  Since x + 0 = x exactly, a sum is bit-identical
// to the reference loop over the same neighbour order.  With --fmad=false
// every FP32 operation rounds like the reference's.
//
// Execution: each lane marches one ray as a small state machine (march,
// bisect, normal, done); every loop iteration each live lane evaluates at most
// one density, so lanes that march and lanes that bisect run the same code
// path together.  128-thread blocks cover 16x8 pixels; a warp owns an 8x4
// tile, so its rays read the same cell rows from L1.

#include <cuda_runtime.h>

#include "fm_internal.cuh"

namespace fm {
namespace {

struct MarchArgs {
    GridDev g;
    KernelDev k;
    float iso, step;
    int max_steps, bisect, skip_mode;
    float cull;  // squared reach in cell units (1 + margin)^2
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
constexpr int kStats = 7;

struct Acc {
    uint32_t evals = 0;
    uint64_t cand = 0;
    uint64_t tested = 0;
    uint32_t skipped = 0;
    bool bad = false;  // an index guard fired (reported through the status word, bit 2)
};

// Location of a sample in the grid: cell and fractional position (cell units).
struct Loc {
    int c[3];
    float u[3];
};

__device__ __forceinline__ bool locate(const GridDev& g, float px, float py, float pz, Loc& L) {
    const float p[3] = {px, py, pz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = (p[a] - g.min[a]) * g.inv;
        float fl = floorf(f);
        if (!(fl >= -2.0f && fl <= (float)g.dims[a] + 1.0f)) return false;
        L.c[a] = (int)fl;
        L.u[a] = f - fl;
    }
    return true;
}

__device__ __forceinline__ float slab_d2(float u, float lo) {
    float d = fmaxf(fmaxf(lo - u, u - (lo + 0.5f)), 0.0f);
    return d * d;
}

// Bit mask over the 24 sub-cells (3 cells x 8) of the row (cy+dy, cz+dz):
// bit 8*i + sub for cell cx-1+i.  Set when the sub-cell box is within reach.
__device__ __forceinline__ uint32_t row_mask(const float ax[6], float yz0, float yz1, float yz2, float yz3, float T) {
    uint32_t m = 0;
    const float yz[4] = {yz0, yz1, yz2, yz3};
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (ax[i] + yz[k] < T) m |= 1u << (8 * (i >> 1) + (i & 1) + 2 * k);
    return m;
}

// Visit, in canonical order, the sorted ranges of every sub-cell within reach
// of the sample; f(b, e) handles particles [b, e).
template <bool STATS, typename F>
__device__ __forceinline__ void for_ranges(const GridDev& g, const Loc& L, float T, Acc& acc, F&& f) {
    float ax[6], ay[6], az[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float lo = -1.0f + 0.5f * (float)i;
        ax[i] = slab_d2(L.u[0], lo);
        ay[i] = slab_d2(L.u[1], lo);
        az[i] = slab_d2(L.u[2], lo);
    }
    const int W = g.dims[0], Hd = g.dims[1], D = g.dims[2];
    uint32_t xvalid = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int x = L.c[0] - 1 + i;
        if (x >= 0 && x < W) xvalid |= 0xffu << (8 * i);
    }
    if (!xvalid) return;
#pragma unroll
    for (int dz = 0; dz < 3; ++dz) {
        const int z = L.c[2] - 1 + dz;
        if (z < 0 || z >= D) continue;
#pragma unroll
        for (int dy = 0; dy < 3; ++dy) {
            const int y = L.c[1] - 1 + dy;
            if (y < 0 || y >= Hd) continue;
            const float yz0 = ay[2 * dy] + az[2 * dz], yz1 = ay[2 * dy + 1] + az[2 * dz];
            const float yz2 = ay[2 * dy] + az[2 * dz + 1], yz3 = ay[2 * dy + 1] + az[2 * dz + 1];
            const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
            // base wraps below 0 when row + cx == 0; then only bits >= 8 are set and
            // base + s wraps back into range.  The index is always formed in uint32
            // before it touches the pointer.
            const uint32_t base = 8u * (row + (uint32_t)L.c[0]) - 8u;
            if (STATS) {
                const int x0 = max(L.c[0] - 1, 0), x1 = min(L.c[0] + 1, W - 1);
                acc.cand += __ldg(g.sub + 8u * (row + x1) + 8u) - __ldg(g.sub + 8u * (row + x0));
            }
            uint32_t m = row_mask(ax, yz0, yz1, yz2, yz3, T) & xvalid;
            while (m) {
                const int s = __ffs(m) - 1;
                const int t = __ffs(~(m >> s)) - 1;  // length of the run of set bits at s
                const uint32_t i0 = base + (uint32_t)s, i1 = i0 + (uint32_t)t;
                if (i1 >= g.nsub) {  // cannot happen for a consistent table; never read past it
                    acc.bad = true;
                    continue;
                }
                const uint32_t b = __ldg(g.sub + i0), e = __ldg(g.sub + i1);
                m &= ~(((1u << t) - 1u) << s);
                if (STATS) acc.tested += e - b;
                f(b, e);
            }
        }
    }
}

// Density at p (canonical order).
template <bool STATS>
__device__ __forceinline__ float density_at(const GridDev& g, const KernelDev& k, const Loc& L, float px, float py,
                                            float pz, float T, Acc& acc) {
    if (STATS) acc.evals++;
    float rho = 0.0f;
    for_ranges<STATS>(g, L, T, acc, [&](uint32_t b, uint32_t e) {
        uint32_t j = b;
        for (; j + 4 <= e; j += 4) {
            const float4 q0 = __ldg(g.pts + j), q1 = __ldg(g.pts + j + 1);
            const float4 q2 = __ldg(g.pts + j + 2), q3 = __ldg(g.pts + j + 3);
            float r0x = q0.x - px, r0y = q0.y - py, r0z = q0.z - pz;
            float r1x = q1.x - px, r1y = q1.y - py, r1z = q1.z - pz;
            float r2x = q2.x - px, r2y = q2.y - py, r2z = q2.z - pz;
            float r3x = q3.x - px, r3y = q3.y - py, r3z = q3.z - pz;
            const float d0 = dot3(r0x, r0y, r0z, r0x, r0y, r0z);
            const float d1 = dot3(r1x, r1y, r1z, r1x, r1y, r1z);
            const float d2 = dot3(r2x, r2y, r2z, r2x, r2y, r2z);
            const float d3 = dot3(r3x, r3y, r3z, r3x, r3y, r3z);
            if (d0 < k.h2) rho = rho + w_in(k, d0);
            if (d1 < k.h2) rho = rho + w_in(k, d1);
            if (d2 < k.h2) rho = rho + w_in(k, d2);
            if (d3 < k.h2) rho = rho + w_in(k, d3);
        }
        for (; j < e; ++j) {
            const float4 q = __ldg(g.pts + j);
            const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
            const float d = dot3(rx, ry, rz, rx, ry, rz);
            if (d < k.h2) rho = rho + w_in(k, d);
        }
    });
    return rho;
}

template <bool STATS>
__device__ __forceinline__ void grad_at(const GridDev& g, const KernelDev& k, float px, float py, float pz, float T,
                                        Acc& acc, float& gx, float& gy, float& gz) {
    gx = gy = gz = 0.0f;
    Loc L;
    if (STATS) acc.evals++;
    if (!locate(g, px, py, pz, L)) return;
    for_ranges<STATS>(g, L, T, acc, [&](uint32_t b, uint32_t e) {
        for (uint32_t j = b; j < e; ++j) {
            const float4 q = __ldg(g.pts + j);
            const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
            const float q2 = dot3(rx, ry, rz, rx, ry, rz);
            if (q2 < k.h2 && q2 > 0.0f) gradw_acc(k, rx, ry, rz, q2, gx, gy, gz);
        }
    });
}

// glm min/max semantics (func_common.inl): min(x,y) = y<x ? y : x, max(x,y) = x<y ? y : x
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }

// The reference's empty-space skip loop (RayMarcher.cpp:284-306), capped.
__device__ __forceinline__ void ref_skip(const GridDev& g, float& px, float& py, float& pz, float sx, float sy,
                                         float sz, unsigned int* status) {
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
    float mx = bx - 2.0f * floorf(bx / 2.0f);
    float mz = bz - 2.0f * floorf(bz / 2.0f);
    float fx = (1.0f < mx) ? 0.0f : 1.0f;
    float fz = (1.0f < mz) ? 0.0f : 1.0f;
    float c = 0.25f + (fx + fz) / 4.0f;
    return make_float4(c, c, c, 0.5f);
}

// composition.frag:132-184, active branch.
__device__ __forceinline__ float4 shade(const MarchArgs& a, int px, int py, bool hit, float hx, float hy, float hz,
                                        float nx, float ny, float nz) {
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

enum Phase : int { kMarch = 0, kBisect = 1, kNormal = 2, kDone = 3 };

template <bool STATS>
__global__ void __launch_bounds__(kThreads) k_march(const MarchArgs a) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = blockIdx.x * kTileW + (warp & 1) * 8 + (lane & 7);
    const int py = blockIdx.y * kTileH + (warp >> 1) * 4 + (lane >> 3);
    const bool valid = px < a.W && py < a.Hh;
    const uint64_t idx = (uint64_t)py * a.W + px;
    Acc acc;
    int phase = kDone;
    bool hit = false, started = false;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f;        // current sample / upper bisection end
    float q0 = 0.f, q1 = 0.f, q2 = 0.f;        // previous sample / lower bisection end
    float sx = 0.f, sy = 0.f, sz = 0.f;
    int i = 0, b = 0;
    if (valid) {
        const float z = a.zbuf[idx];
        if (z != 1.0f) {
            started = true;
            phase = kMarch;
            const float cxp = (float)px * a.twoWinv - 1.0f;
            const float cyp = (float)py * a.twoHinv - 1.0f;
            float wh[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float add0 = a.ipv[0 * 4 + r] * cxp + a.ipv[1 * 4 + r] * cyp;
                float add1 = a.ipv[2 * 4 + r] * z + a.ipv[3 * 4 + r] * 1.0f;
                wh[r] = add0 + add1;
            }
            p0 = wh[0] / wh[3];
            p1 = wh[1] / wh[3];
            p2 = wh[2] / wh[3];
            float dx = p0 - a.cam[0], dy = p1 - a.cam[1], dz = p2 - a.cam[2];
            float inv = 1.0f / sqrtf(dot3(dx, dy, dz, dx, dy, dz));
            sx = a.step * (dx * inv);
            sy = a.step * (dy * inv);
            sz = a.step * (dz * inv);
            q0 = p0; q1 = p1; q2 = p2;
        }
    }
    // one density evaluation per live lane per iteration
    while (phase == kMarch || phase == kBisect) {
        float e0, e1, e2;
        bool eval = false, known = false;
        float rho = 0.0f;
        Loc L;
        if (phase == kMarch) {
            // advance to the next sample that needs its density
            while (i < a.max_steps) {
                p0 = p0 + sx; p1 = p1 + sy; p2 = p2 + sz;
                ++i;
                if (a.skip_mode == FM_SKIP_REFERENCE) ref_skip(a.g, p0, p1, p2, sx, sy, sz, a.status);
                if (!locate(a.g, p0, p1, p2, L)) {
                    if (outside_forever(a.g, p0, p1, p2, sx, sy, sz)) { i = a.max_steps; break; }
                    if (STATS) acc.evals++;
                    known = true;  // no particle within reach: density 0
                    break;
                }
                if (a.skip_mode == FM_SKIP_EXACT && L.c[0] >= 0 && L.c[1] >= 0 && L.c[2] >= 0 &&
                    L.c[0] < a.g.dims[0] && L.c[1] < a.g.dims[1] && L.c[2] < a.g.dims[2]) {
                    const uint32_t c = (uint32_t)L.c[0] + (uint32_t)L.c[1] * (uint32_t)a.g.dims[0] +
                                       (uint32_t)L.c[2] * (uint32_t)a.g.dims[0] * (uint32_t)a.g.dims[1];
                    const uint32_t sc = (L.u[0] >= 0.5f ? 1u : 0u) | (L.u[1] >= 0.5f ? 2u : 0u) | (L.u[2] >= 0.5f ? 4u : 0u);
                    if (__ldg(a.g.bound + 8u * c + sc) < a.iso) {
                        if (STATS) acc.skipped++;
                        q0 = p0; q1 = p1; q2 = p2;
                        continue;
                    }
                }
                eval = true;
                break;
            }
            if (!eval && !known) {  // march ended without a hit
                phase = kDone;
                break;
            }
            e0 = p0; e1 = p1; e2 = p2;
        } else {
            e0 = (q0 + p0) * 0.5f;
            e1 = (q1 + p1) * 0.5f;
            e2 = (q2 + p2) * 0.5f;
            if (!locate(a.g, e0, e1, e2, L)) {
                if (STATS) acc.evals++;
                known = true;
            } else {
                eval = true;
            }
        }
        if (eval) rho = density_at<STATS>(a.g, a.k, L, e0, e1, e2, a.cull, acc);
        const bool inside = rho >= a.iso;
        if (phase == kMarch) {
            if (inside) {
                hit = true;
                b = 0;
                phase = a.bisect > 0 ? kBisect : kNormal;
            } else {
                q0 = p0; q1 = p1; q2 = p2;
            }
        } else {
            if (inside) { p0 = e0; p1 = e1; p2 = e2; }
            else { q0 = e0; q1 = e1; q2 = e2; }
            if (++b >= a.bisect) phase = kNormal;
        }
    }
    float nx = 0.f, ny = 0.f, nz = 0.f;
    if (acc.bad) atomicOr(a.status, 2u);
    if (hit) {
        float gx, gy, gz;
        grad_at<STATS>(a.g, a.k, p0, p1, p2, a.cull, acc, gx, gy, gz);
        float gi = 1.0f / sqrtf(dot3(gx, gy, gz, gx, gy, gz));
        nx = gx * gi; ny = gy * gi; nz = gz * gi;
    }
    if (valid) {
        if (a.pos) a.pos[idx] = hit ? make_float4(p0, p1, p2, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.nrm) a.nrm[idx] = hit ? make_float4(nx, ny, nz, 1.0f) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (a.depth) {
            float d = 0.0f;
            if (hit) {
                float rx = p0 - a.cam[0], ry = p1 - a.cam[1], rz = p2 - a.cam[2];
                d = sqrtf(dot3(rx, ry, rz, rx, ry, rz));
            }
            a.depth[idx] = d;
        }
        if (a.col) a.col[idx] = shade(a, px, py, hit, p0, p1, p2, nx, ny, nz);
    }
    if (STATS) {
        unsigned long long v[kStats] = {valid ? 1ull : 0ull, started ? 1ull : 0ull, hit ? 1ull : 0ull,
                                        (unsigned long long)acc.evals, (unsigned long long)acc.cand,
                                        (unsigned long long)acc.skipped, (unsigned long long)acc.tested};
#pragma unroll
        for (int j = 0; j < kStats; ++j) {
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
    // reach of the support radius in cell units (cell width == support radius),
    // widened to cover the rounding of (p - min) * inv on grids up to 10^6 cells
    int maxdim = s->dims[0] > s->dims[1] ? s->dims[0] : s->dims[1];
    maxdim = maxdim > s->dims[2] ? maxdim : s->dims[2];
    const float reach = 1.0f + 1.0e-3f + 1.0e-6f * (float)maxdim;
    a.cull = reach * reach;
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
