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
//                  bound boxes (an eighth of a cell per axis) whose density
//                  upper bound is below iso are stepped over without
//                  evaluating, so results equal skip-off exactly
//   refinement     bisection between the last outside and first inside sample
//   normal         normalize(sum_j gradW(x_j - p_hit)) (:332-338, Kernel.cpp:34-52)
//   shading        composition.frag:132-184 fused into the epilogue
//
// Summation order is the canonical order: the particles of the 27 cells in
// sorted order (cell, 2x2x2 sub-cell, input index).  Sub-cells out of reach of
// the sample (box distance >= support radius, with a margin for rounding) hold
// only particles with W = 0 and are skipped; every other particle's W is added
// in order.  x + 0 = x exactly, so each sum is bit-identical to the
// reference's sequential loop over the same neighbour order; --fmad=false
// makes every FP32 operation round as the reference's does.
//
// Execution, two passes:
//   k_march       a persistent grid of warps takes 8x4-pixel tiles from an
//                 atomic counter; lane = ray.  Each lane runs a small state
//                 machine (march / bisect / normal / done, `prepare` and
//                 `apply`).  All lanes that need a density sum in the same
//                 iteration share one candidate stream: lanes whose cells lie
//                 in a 2x2x2 cell block are grouped, every cell row of the
//                 group's 4x4x4-cell union is walked once in ascending sorted
//                 order with one broadcast load per particle, and a lane adds
//                 a particle only when its sub-cell is in the lane's own
//                 reach mask, so every lane's sum visits exactly its own
//                 canonical sequence.  When at most 2 lanes are still active,
//                 or after 32 iterations, the remaining rays are pushed to a
//                 long-ray queue with their full state.
//   k_march_long  persistent warps pop queued rays and finish each with all
//                 32 lanes: the reachable sub-cell ranges of the 27 cells are
//                 walked 32 particles at a time (one coalesced load), W is
//                 evaluated in parallel and added to the running sum in lane
//                 order through warp shuffles.
// The 4 float4 outputs are written by whichever pass finishes the ray.

#include <cuda_runtime.h>

#include <cstring>

#include "fm_internal.cuh"

namespace fm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 256;  // 8 warps per block
constexpr int kStats = 12;  // fm_march_stats field order

struct Acc {
    uint32_t evals = 0;
    uint64_t cand = 0;
    uint64_t tested = 0;
    uint64_t streamed = 0;   // shared-stream particles (counted by lane 0 of the warp)
    uint32_t deferred = 0;   // rays handed to the long-ray pass
    uint32_t skipped = 0;
    uint32_t proposed = 0;   // rays that started inside a proposed interval
    uint32_t fallbacks = 0;  // of those, rays restarted as full marches
    uint32_t regrouped = 0;  // rays the first pass handed to the regrouped second pass
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

// Exact-skip bound of the bound box that holds a located sample (1/8 cell per
// axis; u < 1 inside the grid, clamped all the same): no sample in
// the box reaches a density above it, and 0 means no particle lies within the
// support radius of the box.  +inf for a cell outside the grid.
__device__ __forceinline__ float box_bound(const GridDev& g, const Loc& L) {
    if (L.c[0] < 0 || L.c[1] < 0 || L.c[2] < 0 || L.c[0] >= g.dims[0] || L.c[1] >= g.dims[1] || L.c[2] >= g.dims[2])
        return __int_as_float(0x7f800000);
    const uint32_t c = (uint32_t)L.c[0] + (uint32_t)L.c[1] * (uint32_t)g.dims[0] +
                       (uint32_t)L.c[2] * (uint32_t)g.dims[0] * (uint32_t)g.dims[1];
    const uint32_t bx = min((uint32_t)(8.0f * L.u[0]), 7u), by = min((uint32_t)(8.0f * L.u[1]), 7u),
                   bz = min((uint32_t)(8.0f * L.u[2]), 7u);
    return __ldg(g.bound + (uint64_t)kBoundBoxes * c + (bx | (by << 3) | (bz << 6)));
}

// Squared distance (cell units) from fraction u to the half-cell slab [lo, lo + 0.5].
__device__ __forceinline__ float slab_d2(float u, float lo) {
    float d = fmaxf(fmaxf(lo - u, u - (lo + 0.5f)), 0.0f);
    return d * d;
}

// Walk, in canonical order, the particles of the sub-cells within reach of the
// sample at L (warp-uniform: every lane sees the same sequence), packed: per
// row, the reachable sub-cells' particles
// are numbered consecutively (sub-cell order, then sorted order) and handed
// out 32 at a time, lane l taking number v0 + l; f(q, ok) gets the lane's
// particle (ok false past the row's end).  The particles of the next 32 are
// loaded before f runs on the current ones.  Lane l < 24 owns sub-cell l of
// the row (cell cx - 1 + (l >> 3), sub-cell l & 7) and its range; a number's
// owner is found by a binary search over the lanes' running counts.
template <bool STATS, typename F>
__device__ __forceinline__ void for_packed_warp(const GridDev& g, const Loc& L, float T, int lane, Acc& acc, bool cnt,
                                                F&& f) {
    const int W = g.dims[0], Hd = g.dims[1], D = g.dims[2];
    const int ci = lane >> 3, sb = lane & 7;
    const int xl = L.c[0] - 1 + ci;
    const bool lane_ok = lane < 24 && xl >= 0 && xl < W;
    const float dx2 = slab_d2(L.u[0], -1.0f + 0.5f * (float)(2 * ci + (sb & 1)));
#pragma unroll 1
    for (int dz = 0; dz < 3; ++dz) {
        const int z = L.c[2] - 1 + dz;
        if (z < 0 || z >= D) continue;
        const float dz2 = slab_d2(L.u[2], -1.0f + 0.5f * (float)(2 * dz + ((sb >> 2) & 1)));
#pragma unroll 1
        for (int dy = 0; dy < 3; ++dy) {
            const int y = L.c[1] - 1 + dy;
            if (y < 0 || y >= Hd) continue;
            const float dy2 = slab_d2(L.u[1], -1.0f + 0.5f * (float)(2 * dy + ((sb >> 1) & 1)));
            const bool reach = lane_ok && (dx2 + dy2 + dz2 < T);
            const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
            if (STATS && cnt) {  // every row of the 27 cells, reached or not: the reference's candidates
                const int x0 = max(L.c[0] - 1, 0), x1 = min(L.c[0] + 1, W - 1);
                if (x0 <= x1) acc.cand += __ldg(g.sub + 8u * (row + (uint32_t)x1) + 8u) - __ldg(g.sub + 8u * (row + (uint32_t)x0));
            }
            if (!__any_sync(kFull, reach)) continue;
            // base wraps below 0 when row + cx == 0 (then lanes 0-7 are out of the grid);
            // indices are formed in uint32 and loads past the table are never made
            const uint32_t base = 8u * (row + (uint32_t)L.c[0]) - 8u;
            const uint32_t il = base + (uint32_t)lane;
            const uint32_t st = (lane <= 24 && il < g.nsub) ? __ldg(g.sub + il) : 0u;
            const uint32_t en = __shfl_down_sync(kFull, st, 1);
            const uint32_t c = reach ? en - st : 0u;
            uint32_t incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += t;
            }
            const uint32_t excl = incl - c;
            const uint32_t N = __shfl_sync(kFull, incl, 31);
            if (STATS && cnt) acc.tested += N;
            // particle of number v: owner lane = number of lanes whose running count is <= v
            auto particle = [&](uint32_t v) -> uint32_t {
                int o = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const uint32_t it = __shfl_sync(kFull, incl, o + step - 1);
                    if (it <= v) o += step;
                }
                const uint32_t s0 = __shfl_sync(kFull, st, o & 31), e0 = __shfl_sync(kFull, excl, o & 31);
                return s0 + (v - e0);
            };
            uint32_t v = (uint32_t)lane;
            bool ok = v < N;
            uint32_t j = particle(v);
            float4 q = ok ? __ldg(g.pts + j) : make_float4(0.f, 0.f, 0.f, 0.f);
            for (uint32_t v0 = 0; v0 < N; v0 += 32) {
                const uint32_t vn = v0 + 32u + (uint32_t)lane;
                const bool okn = vn < N;
                float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
                if (v0 + 32u < N) {
                    const uint32_t jn = particle(vn);
                    if (okn) qn = __ldg(g.pts + jn);
                }
                f(q, ok);
                q = qn;
                ok = okn;
            }
        }
    }
}

// Add the 32 lanes' terms to acc in lane order, identically on every lane.
// Terms are >= 0 and acc starts at +0, so acc is never -0 and acc + 0 = acc
// exactly: only the nonzero terms need adding.  They are packed in lane order
// into this warp's 32 words of shared memory (padded with +0 to a multiple of
// 4) and added four per 16-byte read, which shortens the dependent chain of
// additions to the number of terms inside the support.
__device__ __forceinline__ float ordered_sum32(float* s, int lane, float w, float acc) {
    const uint32_t m = __ballot_sync(kFull, w != 0.0f);
    const int n = __popc(m);
    __syncwarp();
    if (w != 0.0f) s[__popc(m & ((1u << lane) - 1u))] = w;
    if (lane >= n && lane < ((n + 3) & ~3)) s[lane] = 0.0f;
    __syncwarp();
    const float4* s4 = reinterpret_cast<const float4*>(s);
    for (int i = 0; i < (n + 3) >> 2; ++i) {
        const float4 v = s4[i];
        acc = acc + v.x;
        acc = acc + v.y;
        acc = acc + v.z;
        acc = acc + v.w;
    }
    return acc;
}

// Density at p, identical on every lane (canonical order).  cnt: this lane
// counts the work; red: this warp's 32 words of shared memory.
template <bool STATS>
__device__ __forceinline__ float density_warp(const GridDev& g, const KernelDev& k, const Loc& L, float px, float py,
                                              float pz, float T, int lane, Acc& acc, bool cnt, float* red) {
    if (STATS && cnt) acc.evals++;
    float rho = 0.0f;
    for_packed_warp<STATS>(g, L, T, lane, acc, cnt, [&](const float4& q, bool ok) {
        float w = 0.0f;
        if (ok) {
            const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
            const float d2 = dot3(rx, ry, rz, rx, ry, rz);
            if (d2 < k.h2) w = w_in(k, d2);
        }
        rho = ordered_sum32(red, lane, w, rho);
    });
    return rho;
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

__device__ __forceinline__ void write_pixel(const MarchArgs& a, uint64_t idx, int px, int py, bool hit, float hx,
                                            float hy, float hz, float nx, float ny, float nz) {
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

// ---- per-lane ray state -------------------------------------------------------

enum Phase : int { kMarch = 0, kBisect = 1, kNormal = 2, kDone = 3, kRestart = 4 };

// LEARNED march modes.  kInterval: samples ks+1 .. kf of the plain lattice.
// When that finds no crossing, or its first sample is already inside, the ray
// goes back to its start and marches the prefix 1 .. ks (kPrefixClear /
// kPrefixInside); after the prefix it resumes exactly where the plain march
// would be, without evaluating any sample twice: after kf (samples ks+1 .. kf
// are known outside) or with the crossing at ks+1 (known inside).
enum Mode : int { kWhole = 0, kInterval = 1, kPrefixInside = 2, kPrefixClear = 3 };

struct Ray {
    int phase;
    int i, b;             // march steps taken, bisection steps taken
    float p[3];           // current sample (march) / inside end (bisection)
    float q[3];           // previous sample (march) / outside end (bisection)
    float s[3];           // step
    float e[3];           // pending evaluation point
    int ks, kf;           // proposed interval: samples ks+1 .. kf
    int mode;             // Mode (LEARNED)
};

// Apply the density at the pending point (RayMarcher.cpp:327: hit when rho >= iso).
// LEARNED: a ray marching a proposed interval whose first sample is already
// inside cannot tell whether the crossing lies before the interval: it goes
// back for the prefix.
template <bool LEARNED>
__device__ __forceinline__ void apply(const MarchArgs& a, Ray& r, float rho) {
    const bool inside = rho >= a.iso;
    if (r.phase == kMarch) {
        if (LEARNED && inside && r.mode == kInterval && r.i == r.ks + 1) {
            r.phase = kRestart;
            r.mode = kPrefixInside;
        } else if (inside) {
            r.b = 0;
            r.phase = a.bisect > 0 ? kBisect : kNormal;
        } else {
            r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
        }
    } else {
        if (inside) { r.p[0] = r.e[0]; r.p[1] = r.e[1]; r.p[2] = r.e[2]; }
        else { r.q[0] = r.e[0]; r.q[1] = r.e[1]; r.q[2] = r.e[2]; }
        if (++r.b >= a.bisect) r.phase = kNormal;
    }
}

// Advance a ray to its next density evaluation: march samples are stepped
// (and, for FM_SKIP_EXACT, skipped while their bound box's bound is below iso),
// samples out of reach of every particle get density 0 without a sum.
// Returns true with r.e / L set when a sum is needed, false when the ray left
// the march or bisection phases.
// LEARNED: a ray in a proposed interval that reaches the interval's end (or
// leaves the grid) without a crossing goes back for the prefix (kRestart); a
// ray that finished its prefix resumes the plain march (see Mode).
template <bool STATS, bool LEARNED>
__device__ __forceinline__ bool prepare(const MarchArgs& a, Ray& r, Loc& L, Acc& acc, bool cnt) {
    for (;;) {
        if (r.phase == kMarch) {
            if (LEARNED && r.mode == kInterval && r.i >= r.kf) {
                r.phase = kRestart;
                r.mode = kPrefixClear;
                return false;
            }
            if (LEARNED && r.mode >= kPrefixInside && r.i >= r.ks) {
                if (r.mode == kPrefixInside) {
                    // sample ks+1 is inside: it is the plain march's first crossing
                    r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
                    r.p[0] = r.p[0] + r.s[0];
                    r.p[1] = r.p[1] + r.s[1];
                    r.p[2] = r.p[2] + r.s[2];
                    r.i = r.ks + 1;
                    r.mode = kWhole;
                    r.b = 0;
                    r.phase = a.bisect > 0 ? kBisect : kNormal;
                    continue;
                }
                // samples ks+1 .. kf are outside: go on after kf
                for (int k = r.ks; k < r.kf; ++k) {
                    r.p[0] = r.p[0] + r.s[0];
                    r.p[1] = r.p[1] + r.s[1];
                    r.p[2] = r.p[2] + r.s[2];
                }
                r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
                r.i = r.kf;
                r.mode = kWhole;
                continue;
            }
            if (r.i >= a.max_steps) { r.phase = kDone; return false; }
            r.p[0] = r.p[0] + r.s[0];
            r.p[1] = r.p[1] + r.s[1];
            r.p[2] = r.p[2] + r.s[2];
            ++r.i;
            if (a.skip_mode == FM_SKIP_REFERENCE) ref_skip(a.g, r.p[0], r.p[1], r.p[2], r.s[0], r.s[1], r.s[2], a.status);
            if (zero_density(a.g, r.p[0], r.p[1], r.p[2]) || !locate(a.g, r.p[0], r.p[1], r.p[2], L)) {
                // density exactly 0 here; with iso > 0 no later sample of a ray leaving the
                // zero-density box can hit
                if ((a.iso > 0.0f && leaving_zero_box(a.g, r.p[0], r.p[1], r.p[2], r.s[0], r.s[1], r.s[2])) ||
                    outside_forever(a.g, r.p[0], r.p[1], r.p[2], r.s[0], r.s[1], r.s[2])) {
                    // every later sample has density 0; an interval still needs its prefix
                    r.phase = kDone;
                    if (LEARNED && r.mode == kInterval) {
                        r.phase = kRestart;
                        r.mode = kPrefixClear;
                    }
                    return false;
                }
                if (STATS && cnt) acc.evals++;
                apply<LEARNED>(a, r, 0.0f);
                continue;
            }
            if (a.skip_mode == FM_SKIP_EXACT && box_bound(a.g, L) < a.iso) {
                if (STATS && cnt) acc.skipped++;
                r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
                continue;
            }
            r.e[0] = r.p[0]; r.e[1] = r.p[1]; r.e[2] = r.p[2];
            return true;
        } else if (r.phase == kBisect) {
            r.e[0] = (r.q[0] + r.p[0]) * 0.5f;
            r.e[1] = (r.q[1] + r.p[1]) * 0.5f;
            r.e[2] = (r.q[2] + r.p[2]) * 0.5f;
            if (zero_density(a.g, r.e[0], r.e[1], r.e[2]) || !locate(a.g, r.e[0], r.e[1], r.e[2], L)) {
                if (STATS && cnt) acc.evals++;
                apply<LEARNED>(a, r, 0.0f);
                continue;
            }
            return true;
        }
        return false;
    }
}

// ---- shared candidate stream: lanes are rays ----------------------------------
//
// The lanes that need a sum are grouped so that a group's cells span at most
// 2 per axis; for every cell row of the group's union neighbourhood (4x4 rows,
// 4 cells = 32 sub-cells per row) each lane computes the mask of its own
// reachable sub-cells (only cells within one of its own cell), the warp ORs
// the masks, and all lanes walk the union's sub-cells in ascending order with
// one broadcast load per particle.  A lane adds a particle only when the
// particle's sub-cell is in its own mask, so its sum visits exactly its own
// canonical sequence.

// Own sub-cell reach mask of a lane for cell row (y, z), in union bit
// positions (cell x - (gx - 1)) * 8 + sub, where gx is the group's min cell.
__device__ __forceinline__ uint32_t own_row_mask(const GridDev& g, const Loc& L, const float ax[6], int y, int z, int gx,
                                                 float T) {
    const int dy = y - L.c[1], dz = z - L.c[2];
    if (dy < -1 || dy > 1 || dz < -1 || dz > 1) return 0u;
    const float y0 = slab_d2(L.u[1], (float)dy), y1 = slab_d2(L.u[1], (float)dy + 0.5f);
    const float z0 = slab_d2(L.u[2], (float)dz), z1 = slab_d2(L.u[2], (float)dz + 0.5f);
    const float yz[4] = {y0 + z0, y1 + z0, y0 + z1, y1 + z1};
    uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (ax[i] + yz[k] < T) m |= 1u << (8 * (i >> 1) + (i & 1) + 2 * k);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int x = L.c[0] - 1 + i;
        if (x < 0 || x >= g.dims[0]) m &= ~(0xffu << (8 * i));
    }
    // own cells cx-1..cx+1 sit at union cells (cx - gx) .. (cx - gx + 2)
    return m << (8 * (L.c[0] - gx));
}

// Visit the union stream.  f(pred, b, e): particles [b, e) of one sub-cell,
// pred = this lane's own mask holds it.  `mine`: this lane takes part.
template <bool STATS, typename F>
__device__ __forceinline__ void union_stream(const GridDev& g, bool mine, const Loc& L, float T, Acc& acc, F&& f) {
    float ax[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) ax[i] = slab_d2(L.u[0], -1.0f + 0.5f * (float)i);
    const int W = g.dims[0], Hd = g.dims[1], D = g.dims[2];
    uint32_t pending = __ballot_sync(kFull, mine);
    // Each pass takes the lowest pending lane as leader and groups the lanes
    // whose cells lie in a 2x2x2 block that contains the leader's cell, so
    // every pass retires at least the leader: at most 32 passes.
    for (int pass = 0; pending && pass < 32; ++pass) {
        const bool cand = (pending >> (threadIdx.x & 31)) & 1u;
        const int lead = __ffs(pending) - 1;
        const int lx = __shfl_sync(kFull, L.c[0], lead), ly = __shfl_sync(kFull, L.c[1], lead),
                  lz = __shfl_sync(kFull, L.c[2], lead);
        const bool near = cand && abs(L.c[0] - lx) <= 1 && abs(L.c[1] - ly) <= 1 && abs(L.c[2] - lz) <= 1;
        const int gx = __reduce_min_sync(kFull, near ? L.c[0] : 0x7fffffff);
        const int gy = __reduce_min_sync(kFull, near ? L.c[1] : 0x7fffffff);
        const int gz = __reduce_min_sync(kFull, near ? L.c[2] : 0x7fffffff);
        const bool in = near && L.c[0] - gx <= 1 && L.c[1] - gy <= 1 && L.c[2] - gz <= 1;
        pending &= ~__ballot_sync(kFull, in);
        if (STATS && in) {
            const int x0 = max(L.c[0] - 1, 0), x1 = min(L.c[0] + 1, W - 1);
            if (x0 <= x1)
                for (int z = max(L.c[2] - 1, 0); z <= min(L.c[2] + 1, D - 1); ++z)
                    for (int y = max(L.c[1] - 1, 0); y <= min(L.c[1] + 1, Hd - 1); ++y) {
                        const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
                        acc.cand += __ldg(g.sub + 8u * (row + (uint32_t)x1) + 8u) - __ldg(g.sub + 8u * (row + (uint32_t)x0));
                    }
        }
#pragma unroll 1
        for (int zz = 0; zz < 4; ++zz) {
            const int z = gz - 1 + zz;
            if (z < 0 || z >= D) continue;
#pragma unroll 1
            for (int yy = 0; yy < 4; ++yy) {
                const int y = gy - 1 + yy;
                if (y < 0 || y >= Hd) continue;
                const uint32_t own = in ? own_row_mask(g, L, ax, y, z, gx, T) : 0u;
                uint32_t uni = __reduce_or_sync(kFull, own);
                if (!uni) continue;
                const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
                // base wraps below 0 when row + gx == 0; then only bits >= 8 are set.
                const uint32_t base = 8u * (row + (uint32_t)gx) - 8u;
                // the row's 33 sub-cell starts in one coalesced load: lane l holds
                // start base + l, lane 0 also start base + 32 (indices past the
                // table, including wrapped ones, are never used: their bits are clear)
                const uint32_t il = base + (uint32_t)(threadIdx.x & 31);
                const uint32_t mystart = il < g.nsub ? __ldg(g.sub + il) : 0u;
                const uint32_t i32 = base + 32u;
                const uint32_t start32 = i32 < g.nsub ? __ldg(g.sub + i32) : 0u;
                if ((uni >> 31) && i32 >= g.nsub) acc.bad = true;  // cannot happen for a consistent table
                while (uni) {
                    const int u = __ffs(uni) - 1;
                    uni &= uni - 1u;
                    const uint32_t b = __shfl_sync(kFull, mystart, u);
                    const uint32_t enext = __shfl_sync(kFull, mystart, (u + 1) & 31);
                    const uint32_t e = (u == 31) ? start32 : enext;
                    const bool pred = (own >> u) & 1u;
                    if (STATS && pred) acc.tested += e - b;
                    if (STATS && (threadIdx.x & 31) == 0) acc.streamed += e - b;
                    f(pred, b, e);
                }
            }
        }
    }
    if (pending) acc.bad = true;  // unreachable: every pass retires its leader
}

#ifndef FM_STAGE_TMA
#define FM_STAGE_TMA 0
#endif

#if FM_STAGE_TMA
// Staged variant of the union stream (measured against the plain loads): each
// union row's particle span -- first to last reached sub-cell, contiguous in
// the sorted array -- is copied into the warp's shared memory by
// cp.async.bulk in chunks of kStageCh particles, two buffers per warp, each
// with its own mbarrier; the next chunk of the row is in flight while the
// lanes read the current one.  Waits are bounded: after kStageWaitLimit polls
// the status word gets bit 16 and the chunk is read as it is (the results of
// that launch are then reported as invalid).
constexpr int kStageCh = 128;
constexpr uint32_t kStageWaitLimit = 1u << 22;
__shared__ __align__(128) float4 g_stage[kThreads / 32][2][kStageCh];
__shared__ __align__(8) uint64_t g_stage_bar[kThreads / 32][2];
__shared__ uint32_t g_stage_phase[kThreads / 32];

__device__ __forceinline__ void stage_init() {
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        for (int b = 0; b < 2; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"((uint32_t)__cvta_generic_to_shared(&g_stage_bar[w][b]))
                         : "memory");
        g_stage_phase[w] = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
}

// Lane 0: copy n particles from src into buffer b of this warp.
__device__ __forceinline__ void stage_issue(int w, int b, const float4* src, uint32_t n) {
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&g_stage_bar[w][b]);
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&g_stage[w][b][0]);
    const uint32_t bytes = n * 16u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool stage_wait(int w, int b, uint32_t parity) {
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&g_stage_bar[w][b]);
    for (uint32_t i = 0; i < kStageWaitLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// As union_stream, but f(pred, src, n) gets n particles in shared memory.
template <bool STATS, typename F>
__device__ __forceinline__ void union_stream_staged(const GridDev& g, bool mine, const Loc& L, float T, Acc& acc,
                                                    unsigned int* status, F&& f) {
    float ax[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) ax[i] = slab_d2(L.u[0], -1.0f + 0.5f * (float)i);
    const int W = g.dims[0], Hd = g.dims[1], D = g.dims[2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t ph = g_stage_phase[w];
    uint32_t pending = __ballot_sync(kFull, mine);
    for (int pass = 0; pending && pass < 32; ++pass) {
        const bool cand = (pending >> lane) & 1u;
        const int lead = __ffs(pending) - 1;
        const int lx = __shfl_sync(kFull, L.c[0], lead), ly = __shfl_sync(kFull, L.c[1], lead),
                  lz = __shfl_sync(kFull, L.c[2], lead);
        const bool near = cand && abs(L.c[0] - lx) <= 1 && abs(L.c[1] - ly) <= 1 && abs(L.c[2] - lz) <= 1;
        const int gx = __reduce_min_sync(kFull, near ? L.c[0] : 0x7fffffff);
        const int gy = __reduce_min_sync(kFull, near ? L.c[1] : 0x7fffffff);
        const int gz = __reduce_min_sync(kFull, near ? L.c[2] : 0x7fffffff);
        const bool in = near && L.c[0] - gx <= 1 && L.c[1] - gy <= 1 && L.c[2] - gz <= 1;
        pending &= ~__ballot_sync(kFull, in);
        if (STATS && in) {
            const int x0 = max(L.c[0] - 1, 0), x1 = min(L.c[0] + 1, W - 1);
            if (x0 <= x1)
                for (int z = max(L.c[2] - 1, 0); z <= min(L.c[2] + 1, D - 1); ++z)
                    for (int y = max(L.c[1] - 1, 0); y <= min(L.c[1] + 1, Hd - 1); ++y) {
                        const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
                        acc.cand += __ldg(g.sub + 8u * (row + (uint32_t)x1) + 8u) - __ldg(g.sub + 8u * (row + (uint32_t)x0));
                    }
        }
#pragma unroll 1
        for (int zz = 0; zz < 4; ++zz) {
            const int z = gz - 1 + zz;
            if (z < 0 || z >= D) continue;
#pragma unroll 1
            for (int yy = 0; yy < 4; ++yy) {
                const int y = gy - 1 + yy;
                if (y < 0 || y >= Hd) continue;
                const uint32_t own = in ? own_row_mask(g, L, ax, y, z, gx, T) : 0u;
                const uint32_t uni = __reduce_or_sync(kFull, own);
                if (!uni) continue;
                const uint32_t row = ((uint32_t)z * (uint32_t)Hd + (uint32_t)y) * (uint32_t)W;
                const uint32_t base = 8u * (row + (uint32_t)gx) - 8u;
                const uint32_t il = base + (uint32_t)lane;
                const uint32_t mystart = il < g.nsub ? __ldg(g.sub + il) : 0u;
                const uint32_t i32 = base + 32u;
                const uint32_t start32 = i32 < g.nsub ? __ldg(g.sub + i32) : 0u;
                if ((uni >> 31) && i32 >= g.nsub) acc.bad = true;
                const int first = __ffs(uni) - 1, last = 31 - __clz(uni);
                const uint32_t B = __shfl_sync(kFull, mystart, first);
                const uint32_t nx = __shfl_sync(kFull, mystart, (last + 1) & 31);
                const uint32_t E = last == 31 ? start32 : nx;
                if (E <= B) continue;
                const uint32_t nch = (E - B + kStageCh - 1) / kStageCh;
                if (lane == 0) stage_issue(w, 0, g.pts + B, min(E - B, (uint32_t)kStageCh));
                uint32_t rem = uni;
                int u = __ffs(rem) - 1;
                rem &= rem - 1u;
                uint32_t rb = __shfl_sync(kFull, mystart, u);
                uint32_t rn = __shfl_sync(kFull, mystart, (u + 1) & 31);
                uint32_t re = u == 31 ? start32 : rn;
                bool pred = (own >> u) & 1u;
                bool more = true;
                for (uint32_t kc = 0; kc < nch; ++kc) {
                    const int bf = (int)(kc & 1u);
                    const uint32_t cb = B + kc * (uint32_t)kStageCh;
                    const uint32_t ce = min(E, cb + (uint32_t)kStageCh);
                    if (kc + 1 < nch) {
                        __syncwarp();  // the other buffer's chunk (kc - 1) is read by every lane
                        if (lane == 0)
                            stage_issue(w, bf ^ 1, g.pts + ce, min(E - ce, (uint32_t)kStageCh));
                    }
                    if (!stage_wait(w, bf, (ph >> bf) & 1u)) atomicOr(status, 16u);
                    ph ^= 1u << bf;
                    const float4* buf = &g_stage[w][bf][0];
                    while (more && rb < ce) {
                        const uint32_t j0 = max(rb, cb), j1 = min(re, ce);
                        if (STATS && j1 > j0) {
                            if (pred) acc.tested += j1 - j0;
                            if (lane == 0) acc.streamed += j1 - j0;
                        }
                        if (j1 > j0) f(pred, buf + (j0 - cb), j1 - j0);
                        if (re > ce) break;  // the run goes on in the next chunk
                        if (!rem) {
                            more = false;
                            break;
                        }
                        u = __ffs(rem) - 1;
                        rem &= rem - 1u;
                        rb = __shfl_sync(kFull, mystart, u);
                        rn = __shfl_sync(kFull, mystart, (u + 1) & 31);
                        re = u == 31 ? start32 : rn;
                        pred = (own >> u) & 1u;
                    }
                }
                __syncwarp();  // buffers free before the next row's copy
            }
        }
    }
    if (pending) acc.bad = true;
    if (lane == 0) g_stage_phase[w] = ph;
    __syncwarp();
}
#endif

template <bool STATS>
__device__ __forceinline__ float union_density(const MarchArgs& a, bool mine, const Loc& L, const float e[3], Acc& acc) {
    if (STATS && mine) acc.evals++;
    const float px = e[0], py = e[1], pz = e[2];
    const KernelDev& k = a.k;
    float rho = 0.0f;
#if FM_STAGE_TMA
    union_stream_staged<STATS>(a.g, mine, L, a.cull, acc, a.status, [&](bool pred, const float4* src, uint32_t n) {
        uint32_t j = 0;
        for (; j + 4 <= n; j += 4) {
            const float4 q0 = src[j], q1 = src[j + 1], q2 = src[j + 2], q3 = src[j + 3];
            if (pred) {
                const float r0x = q0.x - px, r0y = q0.y - py, r0z = q0.z - pz;
                const float r1x = q1.x - px, r1y = q1.y - py, r1z = q1.z - pz;
                const float r2x = q2.x - px, r2y = q2.y - py, r2z = q2.z - pz;
                const float r3x = q3.x - px, r3y = q3.y - py, r3z = q3.z - pz;
                const float d0 = dot3(r0x, r0y, r0z, r0x, r0y, r0z);
                const float d1 = dot3(r1x, r1y, r1z, r1x, r1y, r1z);
                const float d2 = dot3(r2x, r2y, r2z, r2x, r2y, r2z);
                const float d3 = dot3(r3x, r3y, r3z, r3x, r3y, r3z);
                if (d0 < k.h2) rho = rho + w_in(k, d0);
                if (d1 < k.h2) rho = rho + w_in(k, d1);
                if (d2 < k.h2) rho = rho + w_in(k, d2);
                if (d3 < k.h2) rho = rho + w_in(k, d3);
            }
        }
        for (; j < n; ++j) {
            const float4 q = src[j];
            if (pred) {
                const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
                const float d = dot3(rx, ry, rz, rx, ry, rz);
                if (d < k.h2) rho = rho + w_in(k, d);
            }
        }
    });
    return rho;
#endif
    union_stream<STATS>(a.g, mine, L, a.cull, acc, [&](bool pred, uint32_t b, uint32_t e_) {
        uint32_t j = b;
        for (; j + 4 <= e_; j += 4) {
            const float4 q0 = __ldg(a.g.pts + j), q1 = __ldg(a.g.pts + j + 1);
            const float4 q2 = __ldg(a.g.pts + j + 2), q3 = __ldg(a.g.pts + j + 3);
            if (pred) {
                const float r0x = q0.x - px, r0y = q0.y - py, r0z = q0.z - pz;
                const float r1x = q1.x - px, r1y = q1.y - py, r1z = q1.z - pz;
                const float r2x = q2.x - px, r2y = q2.y - py, r2z = q2.z - pz;
                const float r3x = q3.x - px, r3y = q3.y - py, r3z = q3.z - pz;
                const float d0 = dot3(r0x, r0y, r0z, r0x, r0y, r0z);
                const float d1 = dot3(r1x, r1y, r1z, r1x, r1y, r1z);
                const float d2 = dot3(r2x, r2y, r2z, r2x, r2y, r2z);
                const float d3 = dot3(r3x, r3y, r3z, r3x, r3y, r3z);
                if (d0 < k.h2) rho = rho + w_in(k, d0);
                if (d1 < k.h2) rho = rho + w_in(k, d1);
                if (d2 < k.h2) rho = rho + w_in(k, d2);
                if (d3 < k.h2) rho = rho + w_in(k, d3);
            }
        }
        if (j < e_) {
            // the last 1-3 particles in one round: their loads issue together
            // (the count is the same on every lane), the sums keep their order
            const uint32_t r = e_ - j;
            const float4 q0 = __ldg(a.g.pts + j);
            const float4 q1 = r > 1u ? __ldg(a.g.pts + j + 1) : q0;
            const float4 q2 = r > 2u ? __ldg(a.g.pts + j + 2) : q0;
            if (pred) {
                const float r0x = q0.x - px, r0y = q0.y - py, r0z = q0.z - pz;
                const float r1x = q1.x - px, r1y = q1.y - py, r1z = q1.z - pz;
                const float r2x = q2.x - px, r2y = q2.y - py, r2z = q2.z - pz;
                const float d0 = dot3(r0x, r0y, r0z, r0x, r0y, r0z);
                const float d1 = dot3(r1x, r1y, r1z, r1x, r1y, r1z);
                const float d2 = dot3(r2x, r2y, r2z, r2x, r2y, r2z);
                if (d0 < k.h2) rho = rho + w_in(k, d0);
                if (r > 1u && d1 < k.h2) rho = rho + w_in(k, d1);
                if (r > 2u && d2 < k.h2) rho = rho + w_in(k, d2);
            }
        }
    });
    return rho;
}

template <bool STATS>
__device__ __forceinline__ void union_grad(const MarchArgs& a, bool mine, const Loc& L, const float e[3], Acc& acc,
                                           float& gx, float& gy, float& gz) {
    if (STATS && mine) acc.evals++;
    const float px = e[0], py = e[1], pz = e[2];
    const KernelDev& k = a.k;
    gx = gy = gz = 0.0f;
    // a particle's term when it lies within the support (and not at p), added in order
    auto term = [&](const float4& q) {
        const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
        const float q2 = dot3(rx, ry, rz, rx, ry, rz);
        if (q2 < k.h2 && q2 > 0.0f) gradw_acc(k, rx, ry, rz, q2, gx, gy, gz);
    };
    union_stream<STATS>(a.g, mine, L, a.cull, acc, [&](bool pred, uint32_t b, uint32_t e_) {
        uint32_t j = b;
        for (; j + 4 <= e_; j += 4) {  // four loads issued together
            const float4 q0 = __ldg(a.g.pts + j), q1 = __ldg(a.g.pts + j + 1);
            const float4 q2 = __ldg(a.g.pts + j + 2), q3 = __ldg(a.g.pts + j + 3);
            if (pred) {
                term(q0);
                term(q1);
                term(q2);
                term(q3);
            }
        }
        if (j < e_) {  // the last 1-3 (the count is the same on every lane)
            const uint32_t r = e_ - j;
            const float4 q0 = __ldg(a.g.pts + j);
            const float4 q1 = r > 1u ? __ldg(a.g.pts + j + 1) : q0;
            const float4 q2 = r > 2u ? __ldg(a.g.pts + j + 2) : q0;
            if (pred) {
                term(q0);
                if (r > 1u) term(q1);
                if (r > 2u) term(q2);
            }
        }
    });
}

// ---- long rays: the whole warp continues one ray ---------------------------------

// Ray start and step of pixel (px, py) with splat depth z (RayMarcher.cpp:268-274).
__device__ __forceinline__ void ray_setup(const MarchArgs& a, int px, int py, float z, float p[3], float s[3]) {
    const float cxp = (float)px * a.twoWinv - 1.0f;
    const float cyp = (float)py * a.twoHinv - 1.0f;
    float wh[4];
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        float add0 = a.ipv[0 * 4 + rr] * cxp + a.ipv[1 * 4 + rr] * cyp;
        float add1 = a.ipv[2 * 4 + rr] * z + a.ipv[3 * 4 + rr] * 1.0f;
        wh[rr] = add0 + add1;
    }
    p[0] = wh[0] / wh[3];
    p[1] = wh[1] / wh[3];
    p[2] = wh[2] / wh[3];
    const float dx = p[0] - a.cam[0], dy = p[1] - a.cam[1], dz = p[2] - a.cam[2];
    const float inv = 1.0f / sqrtf(dot3(dx, dy, dz, dx, dy, dz));
    s[0] = a.step * (dx * inv);
    s[1] = a.step * (dy * inv);
    s[2] = a.step * (dz * inv);
}

// Long-ray queue entry: 4 float4 = {pixel, phase | mode << 8, i, b}, {p, ks}, {q, kf}, {e, view}
// (e: the pending evaluation point).  The step is recomputed from the pixel.
struct Queue {
    float4* buf;          // 4 float4 per entry
    unsigned int* tail;   // entries reserved
    unsigned int cap;
};

__device__ __forceinline__ void push_long(const Queue& q, uint32_t slot, uint32_t idx, uint32_t view, const Ray& r) {
    float4* d = q.buf + 4ull * slot;
    d[0] = make_float4(__uint_as_float(idx), __int_as_float(r.phase | (r.mode << 8)), __int_as_float(r.i),
                       __int_as_float(r.b));
    d[1] = make_float4(r.p[0], r.p[1], r.p[2], __int_as_float(r.ks));
    d[2] = make_float4(r.q[0], r.q[1], r.q[2], __int_as_float(r.kf));
    d[3] = make_float4(r.e[0], r.e[1], r.e[2], __uint_as_float(view));
}

// View of a batch tile: the largest v with pfx[v] <= t (pfx[0] = 0, ascending).
__device__ __forceinline__ int find_view(const uint32_t* __restrict__ pfx, int nviews, uint32_t t) {
    int lo = 0, hi = nviews - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pfx + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Sum of gradW at p (canonical order) with the whole warp, identical on every lane.
template <bool STATS>
__device__ __forceinline__ void grad_warp(const GridDev& g, const KernelDev& k, float px, float py, float pz, float T,
                                          int lane, Acc& acc, bool cnt, float* red, float& gx, float& gy, float& gz) {
    gx = gy = gz = 0.0f;
    Loc L;
    if (STATS && cnt) acc.evals++;
    if (!locate(g, px, py, pz, L)) return;
    for_packed_warp<STATS>(g, L, T, lane, acc, cnt, [&](const float4& q, bool ok) {
        {
            float tx = 0.0f, ty = 0.0f, tz = 0.0f;
            if (ok) {
                const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
                const float q2 = dot3(rx, ry, rz, rx, ry, rz);
                if (q2 < k.h2 && q2 > 0.0f) gradw_term(k, rx, ry, rz, q2, tx, ty, tz);
            }
            // in lane order, as ordered_sum32 (components never become -0)
            __syncwarp();
            red[lane] = tx;
            red[32 + lane] = ty;
            red[64 + lane] = tz;
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
                const float4 vx = *reinterpret_cast<const float4*>(red + i);
                const float4 vy = *reinterpret_cast<const float4*>(red + 32 + i);
                const float4 vz = *reinterpret_cast<const float4*>(red + 64 + i);
                gx = gx + vx.x; gy = gy + vy.x; gz = gz + vz.x;
                gx = gx + vx.y; gy = gy + vy.y; gz = gz + vz.y;
                gx = gx + vx.z; gy = gy + vy.z; gz = gz + vz.z;
                gx = gx + vx.w; gy = gy + vy.w; gz = gz + vz.w;
            }
        }
    });
}

// One 32-pixel tile of view `a` (lane = ray).  `view` tags the rays this
// warp defers to the long-ray queue.
// LEARNED: send a ray back to its start for the prefix of its interval.
template <bool STATS>
__device__ __forceinline__ void restart(const MarchArgs& a, Ray& r, int px, int py, uint64_t idx, Acc& acc, bool cnt) {
    ray_setup(a, px, py, a.zbuf[idx], r.p, r.s);
    r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
    r.i = 0;
    r.b = 0;
    r.phase = kMarch;
    if (STATS && cnt) acc.fallbacks++;
}

// Advance to the next sum, restarting rays whose proposed interval failed.
template <bool STATS, bool LEARNED>
__device__ __forceinline__ bool advance(const MarchArgs& a, Ray& r, Loc& L, int px, int py, uint64_t idx, Acc& acc,
                                        bool cnt) {
    if (LEARNED && r.phase == kRestart) restart<STATS>(a, r, px, py, idx, acc, cnt);
    bool need = (r.phase == kMarch || r.phase == kBisect) && prepare<STATS, LEARNED>(a, r, L, acc, cnt);
    if (LEARNED && !need && r.phase == kRestart) {
        restart<STATS>(a, r, px, py, idx, acc, cnt);
        need = prepare<STATS, LEARNED>(a, r, L, acc, cnt);
    }
    return need;
}

// The lanes-are-rays loop: every iteration each active lane advances its ray
// to its next density sum, and the warp computes all sums through one shared
// candidate stream.  `pending`: the lane starts with a prepared evaluation
// point (a ray resumed from a queue).  After `cap` iterations, or once at most
// a.defer_lanes rays are left, the remaining rays go to queue q (rays that find
// it full stay).  Returns true when this lane's ray was queued.
template <bool STATS, bool LEARNED>
__device__ __forceinline__ bool run_lanes(const MarchArgs& a, const Queue& q, Ray& r, Loc& L, bool pending, int px,
                                          int py, uint64_t idx, uint32_t view, int cap, bool to_regroup, int lane,
                                          Acc& acc) {
    int iters = 0;
    bool deferred = false, keep = false;
    for (;;) {
        bool need;
        if (pending) {
            pending = false;
            need = locate(a.g, r.e[0], r.e[1], r.e[2], L);
            if (!need) {  // a prepared point is always inside the evaluation range; be safe anyway
                apply<LEARNED>(a, r, 0.0f);
                need = advance<STATS, LEARNED>(a, r, L, px, py, idx, acc, true);
            }
        } else {
            need = advance<STATS, LEARNED>(a, r, L, px, py, idx, acc, true);
        }
        uint32_t act = __ballot_sync(kFull, need);
        if (!act) break;
        if (!keep && (__popc(act) <= a.defer_lanes || iters >= cap)) {
            // Few rays left, or rays that march long (grazing the surface): hand
            // them on instead of keeping this warp busy with a sparse, scattered
            // set of rays.  Rays that find the queue full stay here, and the
            // warp stops deferring.
            const uint32_t base = (lane == 0) ? atomicAdd(q.tail, (unsigned)__popc(act)) : 0u;
            const uint32_t slot = __shfl_sync(kFull, base, 0) + __popc(act & ((1u << lane) - 1u));
            if (need && slot < q.cap) {
                push_long(q, slot, (uint32_t)idx, view, r);
                deferred = true;
                need = false;
                r.phase = kDone;
                if (STATS) {
                    if (to_regroup) acc.regrouped++;
                    else acc.deferred++;
                }
            }
            act = __ballot_sync(kFull, need);
            if (!act) break;
            keep = true;
        }
        const float rho = union_density<STATS>(a, need, L, r.e, acc);
        if (need) apply<LEARNED>(a, r, rho);
        ++iters;
    }
    return deferred;
}

// Normals of the lanes' hit rays (shared stream), then their pixels.
template <bool STATS>
__device__ __forceinline__ void finish_lanes(const MarchArgs& a, const Ray& r, bool live, uint64_t idx, int px, int py,
                                             Acc& acc, uint64_t& hits) {
    const bool hit = live && r.phase == kNormal;
    Loc Lh;
    Lh.c[0] = Lh.c[1] = Lh.c[2] = 0;
    Lh.u[0] = Lh.u[1] = Lh.u[2] = 0.0f;
    const bool gn = hit && locate(a.g, r.p[0], r.p[1], r.p[2], Lh);
    if (STATS && hit && !gn) acc.evals++;
    float gx = 0.f, gy = 0.f, gz = 0.f;
    if (__any_sync(kFull, gn)) union_grad<STATS>(a, gn, Lh, r.p, acc, gx, gy, gz);
    float n0 = 0.f, n1 = 0.f, n2 = 0.f;
    if (hit) {
        const float gi = 1.0f / sqrtf(dot3(gx, gy, gz, gx, gy, gz));
        n0 = gx * gi;
        n1 = gy * gi;
        n2 = gz * gi;
        if (STATS) hits++;
    }
    if (live) write_pixel(a, idx, px, py, hit, r.p[0], r.p[1], r.p[2], n0, n1, n2);
}

template <bool STATS, bool LEARNED>
__device__ __forceinline__ void march_tile(const MarchArgs& a, const Queue& q, bool to_regroup, unsigned tile,
                                           uint32_t view, int lane, Acc& acc, uint64_t& rays, uint64_t& started_n,
                                           uint64_t& hits) {
    const int tw = 1 << a.tw_log2;
    const int tx = (int)(tile % (unsigned)a.tiles_x), ty = (int)(tile / (unsigned)a.tiles_x);
    const int px = tx * tw + (lane & (tw - 1));
    const int py = ty * (32 >> a.tw_log2) + (lane >> a.tw_log2);
    const bool valid = px < a.W && py < a.Hh;
    const uint64_t idx = (uint64_t)py * (uint64_t)a.W + (uint64_t)px;
    const float z = valid ? a.zbuf[idx] : 1.0f;
    Ray r;
    r.phase = kDone;
    r.i = r.b = 0;
    r.ks = 0;
    r.kf = -1;
    r.mode = kWhole;
    if (valid && z != 1.0f) {
        ray_setup(a, px, py, z, r.p, r.s);
        if (LEARNED && a.ivl) {  // a batch may mix views with and without a proposal
            // start at sample ks of the plain march (the same FP32 additions),
            // evaluate samples ks+1 .. kf
            const int2 iv = a.ivl[idx];
            if (iv.x >= 1 && iv.x < iv.y && iv.y <= a.max_steps) {
                for (int k = 0; k < iv.x; ++k) {
                    r.p[0] = r.p[0] + r.s[0];
                    r.p[1] = r.p[1] + r.s[1];
                    r.p[2] = r.p[2] + r.s[2];
                }
                r.i = iv.x;
                r.ks = iv.x;
                r.kf = iv.y;
                r.mode = kInterval;
                if (STATS) acc.proposed++;
            }
        }
        r.q[0] = r.p[0]; r.q[1] = r.p[1]; r.q[2] = r.p[2];
        r.phase = kMarch;
    } else {
        r.p[0] = r.p[1] = r.p[2] = 0.0f;
        r.q[0] = r.q[1] = r.q[2] = 0.0f;
        r.s[0] = r.s[1] = r.s[2] = 0.0f;
    }
    r.e[0] = r.e[1] = r.e[2] = 0.0f;
    if (STATS && valid) { rays++; if (z != 1.0f) started_n++; }
    Loc L;
    L.c[0] = L.c[1] = L.c[2] = 0;
    L.u[0] = L.u[1] = L.u[2] = 0.0f;
    const bool deferred = run_lanes<STATS, LEARNED>(a, q, r, L, false, px, py, idx, view, a.cap, to_regroup, lane, acc);
    // deferred rays are finished (and written) by a later pass
    finish_lanes<STATS>(a, r, valid && !deferred, idx, px, py, acc, hits);
}

// Ray state of a queue entry (the step comes from the pixel: ray_setup).
__device__ __forceinline__ void load_entry(const float4* __restrict__ d, Ray& r, uint32_t& idx, uint32_t& view) {
    const float4 w0 = d[0], w1 = d[1], w2 = d[2], w3 = d[3];
    idx = __float_as_uint(w0.x);
    r.phase = __float_as_int(w0.y) & 0xff;
    r.mode = __float_as_int(w0.y) >> 8;
    r.i = __float_as_int(w0.z);
    r.b = __float_as_int(w0.w);
    r.p[0] = w1.x; r.p[1] = w1.y; r.p[2] = w1.z;
    r.q[0] = w2.x; r.q[1] = w2.y; r.q[2] = w2.z;
    r.e[0] = w3.x; r.e[1] = w3.y; r.e[2] = w3.z;
    r.ks = __float_as_int(w1.w);
    r.kf = __float_as_int(w2.w);
    view = __float_as_uint(w3.w);
}

__device__ __forceinline__ void flush_stats(const MarchArgs& a, int lane, const Acc& acc, uint64_t rays,
                                            uint64_t started_n, uint64_t hits, bool warp_sum) {
    unsigned long long v[kStats] = {rays, started_n, hits, (unsigned long long)acc.evals,
                                    (unsigned long long)acc.cand, (unsigned long long)acc.skipped,
                                    (unsigned long long)acc.tested, (unsigned long long)acc.streamed,
                                    (unsigned long long)acc.deferred, (unsigned long long)acc.proposed,
                                    (unsigned long long)acc.fallbacks, (unsigned long long)acc.regrouped};
#pragma unroll
    for (int j = 0; j < kStats; ++j) {
        unsigned long long x = v[j];
        if (warp_sum) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
        }
        if (lane == 0 && x) atomicAdd(a.stats + j, x);
    }
}

// Shared-stream pass.  Persistent warps take `a.claim` tiles per atomic from
// the launch's counter.  BATCH: `a` holds the launch-wide fields and the total
// tile count; tile t belongs to view find_view(tile_pfx, t) of `views`.
// Occupancy measured per instantiation: the plain march runs fastest with 3
// blocks of up to 80 registers per SM, the learned one with 4 of 64 (it
// spills, yet at 1080p 8.14 ms against 8.70 ms with 3 blocks of 80).
template <bool STATS, bool BATCH, bool LEARNED>
__global__ void __launch_bounds__(kThreads, LEARNED ? 4 : 3)
    k_march(const MarchArgs a, const MarchArgs* __restrict__ views, const uint32_t* __restrict__ tile_pfx, int nviews) {
    const int lane = threadIdx.x & 31;
#if FM_STAGE_TMA
    stage_init();
#endif
    Acc acc;
    uint64_t rays = 0, started_n = 0, hits = 0;
    const unsigned total = (unsigned)a.ntiles, claim = (unsigned)a.claim;
    const Queue q{a.longq, a.q_tail, a.q_cap};
    const bool to_regroup = a.order != nullptr;
    for (;;) {
        unsigned t0 = 0;
        if (lane == 0) t0 = atomicAdd(a.tile_counter, claim);
        t0 = __shfl_sync(kFull, t0, 0);
        if (t0 >= total) break;
        const unsigned t1 = min(t0 + claim, total);
        for (unsigned t = t0; t < t1; ++t) {
            if (BATCH) {
                const int v = find_view(tile_pfx, nviews, t);
                march_tile<STATS, LEARNED>(views[v], q, to_regroup, t - __ldg(tile_pfx + v), (uint32_t)v, lane, acc,
                                           rays, started_n, hits);
            } else {
                march_tile<STATS, LEARNED>(a, q, to_regroup, t, 0u, lane, acc, rays, started_n, hits);
            }
        }
    }
    if (acc.bad) atomicOr(a.status, 2u);
    if (STATS) flush_stats(a, lane, acc, rays, started_n, hits, true);
}

// ---- regrouped second pass --------------------------------------------------------
//
// The rays the first pass handed on are sorted by the first-pass tile of their
// pixel (a counting sort: tiles are the keys, so rays of neighbouring tiles
// end up next to each other), then marched again 32 to a warp with the same
// shared-stream loop: full warps of rays from the same part of the image
// instead of the few scattered rays each first-pass warp had left.  What this
// pass hands on goes to the warp-per-ray pass.

template <bool BATCH>
__device__ __forceinline__ uint32_t queue_key(const MarchArgs& a, const MarchArgs* __restrict__ views,
                                              const uint32_t* __restrict__ tile_pfx, const float4* __restrict__ d) {
    const float4 w0 = d[0], w3 = d[3];
    const uint32_t idx = __float_as_uint(w0.x);
    uint32_t base = 0;
    int W = a.W, tiles_x = a.tiles_x, lg = a.tw_log2;
    if (BATCH) {
        const uint32_t v = __float_as_uint(w3.w);
        base = __ldg(tile_pfx + v);
        W = views[v].W;
        tiles_x = views[v].tiles_x;
    }
    const uint32_t px = idx % (uint32_t)W, py = idx / (uint32_t)W;
    return base + (py / (uint32_t)(32 >> lg)) * (uint32_t)tiles_x + (px >> lg);
}

template <bool BATCH>
__global__ void k_queue_hist(const MarchArgs a, const MarchArgs* __restrict__ views,
                             const uint32_t* __restrict__ tile_pfx) {
    const unsigned n = min(*(volatile unsigned int*)a.q_tail, a.q_cap);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        atomicAdd(a.keys + queue_key<BATCH>(a, views, tile_pfx, a.longq + 4ull * k), 1u);
}

template <bool BATCH>
__global__ void k_queue_scatter(const MarchArgs a, const MarchArgs* __restrict__ views,
                                const uint32_t* __restrict__ tile_pfx) {
    const unsigned n = min(*(volatile unsigned int*)a.q_tail, a.q_cap);
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t pos = atomicAdd(a.keys + queue_key<BATCH>(a, views, tile_pfx, a.longq + 4ull * k), 1u);
        a.order[pos] = k;
    }
}

template <bool STATS, bool BATCH, bool LEARNED>
__global__ void __launch_bounds__(kThreads, 4) k_regroup(const MarchArgs a, const MarchArgs* __restrict__ views) {
    const int lane = threadIdx.x & 31;
#if FM_STAGE_TMA
    stage_init();
#endif
    Acc acc;
    uint64_t hits = 0;
    const unsigned n = min(*(volatile unsigned int*)a.q_tail, a.q_cap);
    const unsigned groups = (n + 31) / 32;
    const Queue q2{a.longq2, a.q2_tail, a.q_cap};
    for (;;) {
        unsigned g = 0;
        if (lane == 0) g = atomicAdd(a.grp_counter, 1u);
        g = __shfl_sync(kFull, g, 0);
        if (g >= groups) break;
        const unsigned j = g * 32 + (unsigned)lane;
        bool have = j < n;
        Ray r;
        r.phase = kDone;
        r.i = r.b = r.ks = 0;
        r.kf = -1;
        r.mode = kWhole;
        r.p[0] = r.p[1] = r.p[2] = 0.0f;
        r.q[0] = r.q[1] = r.q[2] = 0.0f;
        r.e[0] = r.e[1] = r.e[2] = 0.0f;
        r.s[0] = r.s[1] = r.s[2] = 0.0f;
        uint32_t idx = 0, view = 0;
        if (have) load_entry(a.longq + 4ull * a.order[j], r, idx, view);
        // a warp marches rays of one view: lanes of another view (only where the
        // sorted list crosses a view boundary) go straight to the next queue
        const uint32_t v0 = __shfl_sync(kFull, view, 0);
        if (BATCH && have && view != v0) {
            const uint32_t slot = atomicAdd(a.q2_tail, 1u);
            if (slot < a.q_cap) push_long(q2, slot, idx, view, r);
            if (STATS) acc.deferred++;
            have = false;
            r.phase = kDone;  // the ray is the long-ray pass's now: it must not march here
        }
        const MarchArgs& av = BATCH ? views[v0] : a;
        const int px = have ? (int)(idx % (uint32_t)av.W) : 0, py = have ? (int)(idx / (uint32_t)av.W) : 0;
        if (have) {
            float p0[3];
            ray_setup(av, px, py, av.zbuf[idx], p0, r.s);
        }
        Loc L;
        L.c[0] = L.c[1] = L.c[2] = 0;
        L.u[0] = L.u[1] = L.u[2] = 0.0f;
        const bool deferred =
            run_lanes<STATS, LEARNED>(av, q2, r, L, have, px, py, idx, v0, a.cap2, false, lane, acc);
        finish_lanes<STATS>(av, r, have && !deferred, idx, px, py, acc, hits);
    }
    if (acc.bad) atomicOr(a.status, 2u);
    if (STATS) flush_stats(a, lane, acc, 0, 0, hits, true);
}

// Finish one queued ray with the whole warp and write its pixel.
template <bool STATS, bool LEARNED>
__device__ __forceinline__ void finish_long(const MarchArgs& a, uint32_t idx, Ray& r, int lane, Acc& acc,
                                            uint64_t& hits, float* red) {
    const int px = (int)(idx % (uint32_t)a.W), py = (int)(idx / (uint32_t)a.W);
    float p0[3];
    ray_setup(a, px, py, a.zbuf[idx], p0, r.s);
    const bool cnt = lane == 0;
    Loc L;
    bool need = locate(a.g, r.e[0], r.e[1], r.e[2], L);  // the pending point was prepared
    while (need) {
        const float rho = density_warp<STATS>(a.g, a.k, L, r.e[0], r.e[1], r.e[2], a.cull, lane, acc, cnt, red);
        apply<LEARNED>(a, r, rho);
        need = advance<STATS, LEARNED>(a, r, L, px, py, idx, acc, cnt);
    }
    const bool hit = r.phase == kNormal;
    float n0 = 0.f, n1 = 0.f, n2 = 0.f;
    if (hit) {
        float gx, gy, gz;
        grad_warp<STATS>(a.g, a.k, r.p[0], r.p[1], r.p[2], a.cull, lane, acc, cnt, red, gx, gy, gz);
        const float gi = 1.0f / sqrtf(dot3(gx, gy, gz, gx, gy, gz));
        n0 = gx * gi;
        n1 = gy * gi;
        n2 = gz * gi;
    }
    if (lane == 0) {
        write_pixel(a, idx, px, py, hit, r.p[0], r.p[1], r.p[2], n0, n1, n2);
        if (STATS && hit) hits++;
    }
}

// Long-ray pass: persistent warps take deferred rays one at a time and finish
// them with all 32 lanes (density_warp / grad_warp), then write the pixel.
template <bool STATS, bool BATCH, bool LEARNED>
__global__ void __launch_bounds__(kThreads) k_march_long(const MarchArgs a, const MarchArgs* __restrict__ views,
                                                         const float4* __restrict__ buf,
                                                         const unsigned int* __restrict__ tail,
                                                         unsigned int* __restrict__ head) {
    __shared__ __align__(16) float red_all[kThreads / 32][96];
    float* red = red_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    Acc acc;
    uint64_t hits = 0;
    const unsigned total = min(*(volatile const unsigned int*)tail, a.q_cap);
    for (;;) {
        unsigned k = 0;
        if (lane == 0) k = atomicAdd(head, 1u);
        k = __shfl_sync(kFull, k, 0);
        if (k >= total) break;
        Ray r;
        uint32_t idx, view;
        load_entry(buf + 4ull * k, r, idx, view);
        if (BATCH) finish_long<STATS, LEARNED>(views[view], idx, r, lane, acc, hits, red);
        else finish_long<STATS, LEARNED>(a, idx, r, lane, acc, hits, red);
    }
    if (acc.bad) atomicOr(a.status, 2u);
    if (STATS) {
        acc.streamed = 0;
        acc.deferred = 0;
        acc.proposed = 0;
        acc.regrouped = 0;
        flush_stats(a, lane, acc, 0, 0, hits, false);
    }
}
}  // namespace

MarchArgs march_view_args(const fm_scene* s, const fm_camera* cam, const fm_march_params* p, const MarchOutDev& o,
                          const TileConfig& cfg) {
    MarchArgs a{};
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
    a.tw_log2 = cfg.tw_log2;
    a.claim = cfg.claim;
    // measured optima at 1080p: 12 sums when the march reads the refined
    // (eighth-cell) bound table (7.51 ms against 8.23 ms at 15; the 640x480
    // dam break 1.89 against 2.07 ms), 15 without the exact skip and on a
    // first level alone, which leaves more rays with long runs of sums (12
    // would defer 162k rays: 11.0 ms against 9.9 ms for the frame)
    a.cap = cfg.cap > 0 ? cfg.cap : ((p->skip_mode == FM_SKIP_EXACT && s->bound_fine) ? 12 : 15);
    a.defer_lanes = cfg.lanes;
    a.cap2 = cfg.cap2;
    a.order = nullptr;
    const int tw = 1 << cfg.tw_log2, th = 32 >> cfg.tw_log2;
    a.tiles_x = (cam->width + tw - 1) / tw;
    a.ntiles = a.tiles_x * ((cam->height + th - 1) / th);
    a.twoWinv = 2.0f / (float)cam->width;
    a.twoHinv = 2.0f / (float)cam->height;
    a.zbuf = o.start_depth;
    a.ivl = o.ivl;
    a.pos = o.pos;
    a.nrm = o.nrm;
    a.depth = o.depth;
    a.col = o.col;
    return a;
}

namespace {

template <bool STATS, bool BATCH, bool LEARNED>
int launch_variant(fm_ctx* ctx, const MarchArgs& a, const MarchArgs* d_views, const uint32_t* d_tile_pfx, int nviews,
                   cudaStream_t st) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_march<STATS, BATCH, LEARNED>, kThreads, 0);
    if (per_sm < 1) per_sm = 1;
    int blocks = ctx->sm_count * per_sm;
    const int warps_needed = (a.ntiles + a.claim - 1) / a.claim;
    const int max_blocks = (warps_needed + kThreads / 32 - 1) / (kThreads / 32);
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks < 1) blocks = 1;
    k_march<STATS, BATCH, LEARNED><<<blocks, kThreads, 0, st>>>(a, d_views, d_tile_pfx, nviews);
    FM_CUDA(ctx, cudaGetLastError());
    const float4* lbuf = a.longq;
    const unsigned int* ltail = a.q_tail;
    unsigned int* lhead = a.q_head;
    if (a.order) {
        // regroup: counting sort of the queued rays by first-pass tile, second pass
        const unsigned sblocks = (unsigned)ctx->sm_count * 4;
        FM_CUDA(ctx, cudaMemsetAsync(a.keys, 0, ((size_t)a.ntiles + 1) * sizeof(uint32_t), st));
        k_queue_hist<BATCH><<<sblocks, 256, 0, st>>>(a, d_views, d_tile_pfx);
        scan_exclusive(a.keys, a.keys, (uint64_t)a.ntiles + 1, a.scan_tmp, st);
        k_queue_scatter<BATCH><<<sblocks, 256, 0, st>>>(a, d_views, d_tile_pfx);
        int rg_per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rg_per_sm, k_regroup<STATS, BATCH, LEARNED>, kThreads, 0);
        if (rg_per_sm < 1) rg_per_sm = 1;
        k_regroup<STATS, BATCH, LEARNED><<<ctx->sm_count * rg_per_sm, kThreads, 0, st>>>(a, d_views);
        FM_CUDA(ctx, cudaGetLastError());
        lbuf = a.longq2;
        ltail = a.q2_tail;
        lhead = a.q2_head;
    }
    int long_per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&long_per_sm, k_march_long<STATS, BATCH, LEARNED>, kThreads, 0);
    if (long_per_sm < 1) long_per_sm = 1;
    k_march_long<STATS, BATCH, LEARNED><<<ctx->sm_count * long_per_sm, kThreads, 0, st>>>(a, d_views, lbuf, ltail,
                                                                                          lhead);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace

int launch_march_kernels(fm_ctx* ctx, const MarchArgs& a, const MarchArgs* d_views, const uint32_t* d_tile_pfx,
                         int nviews, cudaStream_t st) {
    const bool stats = a.stats != nullptr, batch = nviews > 0, learned = a.ivl != nullptr;
    const int k = (stats ? 4 : 0) | (batch ? 2 : 0) | (learned ? 1 : 0);
    switch (k) {
        case 0: return launch_variant<false, false, false>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 1: return launch_variant<false, false, true>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 2: return launch_variant<false, true, false>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 3: return launch_variant<false, true, true>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 4: return launch_variant<true, false, false>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 5: return launch_variant<true, false, true>(ctx, a, d_views, d_tile_pfx, nviews, st);
        case 6: return launch_variant<true, true, false>(ctx, a, d_views, d_tile_pfx, nviews, st);
        default: return launch_variant<true, true, true>(ctx, a, d_views, d_tile_pfx, nviews, st);
    }
}

namespace {

// DiskRenderer::ComputeDensity (DiskRenderer.cpp:180-193): density at
// arbitrary points, thread per point, the 27 cells in canonical order (9 rows
// of 3 contiguous cells).  Bit-identical to the march's sums at the same point.
__global__ void k_density_probe(const GridDev g, const KernelDev k, const float* __restrict__ xyz, uint64_t n,
                                uint32_t stride, float* __restrict__ out) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float px = xyz[i * stride], py = xyz[i * stride + 1], pz = xyz[i * stride + 2];
    float rho = 0.0f;
    int c[3];
    if (sample_cell(g, px, py, pz, c[0], c[1], c[2])) {
        const int x0 = max(c[0] - 1, 0), x1 = min(c[0] + 1, g.dims[0] - 1);
        for (int z = max(c[2] - 1, 0); z <= min(c[2] + 1, g.dims[2] - 1); ++z)
            for (int y = max(c[1] - 1, 0); y <= min(c[1] + 1, g.dims[1] - 1); ++y) {
                if (x0 > x1) continue;
                const uint32_t row = ((uint32_t)z * (uint32_t)g.dims[1] + (uint32_t)y) * (uint32_t)g.dims[0];
                const uint32_t b = __ldg(g.sub + 8u * (row + (uint32_t)x0));
                const uint32_t e = __ldg(g.sub + 8u * (row + (uint32_t)x1) + 8u);
                for (uint32_t j = b; j < e; ++j) {
                    const float4 q = __ldg(g.pts + j);
                    const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
                    const float d = dot3(rx, ry, rz, rx, ry, rz);
                    if (d < k.h2) rho = rho + w_in(k, d);
                }
            }
    }
    out[i] = rho;
}

}  // namespace

namespace {

// ---- anisotropic march (RayMarcher.cpp:346-423, WPCA :114-249, Kernel.cpp:55-107) ----
//
// Warp per ray.  Every sample (march, bisection, normal) runs the reference's
// WPCA over the particles within the extended radius (the 5x5x5 cells around
// the sample): CubicKernel weights 1 - (|r| / Hext)^3, weighted mean,
// weighted covariance, eigen-decomposition (cyclic Jacobi in FP32), the
// [YT13] eq. 15 clamp (k_n, k_r, k_s, N_eps), G = (1/H) R Sigma^-1 R^T; then
// the anisotropic density sum over the particles within H.  Sums are per lane
// and reduced over the warp (a fixed butterfly), so the result agrees with the
// CPU restatement to rounding, not bit for bit (the eigen solver's square
// roots and the summation order differ).

struct AnisoDev {
    float reach2_ext, reach2;      // squared sub-cell reach (cell units) of Hext and H, with a rounding margin
    float hext, hext2, hext_inv;   // extended radius
    float h, h2, hinv, sig;        // AnisotropicKernel(H): sig = 8 / pi
    float k_n, k_r, k_s;
    int n_eps;
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// Symmetric 3x3 eigen-decomposition by cyclic Jacobi rotations in FP32 (the
// reference solves in FP32 too; FP64 runs at a small fraction of the FP32 rate
// on this part).  Stops when the off-diagonal mass is below 1e-14 of the
// diagonal's, after at most 16 sweeps.
__device__ __forceinline__ void eig3_jacobi(float A[3][3], float w[3], float V[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0f : 0.0f;
    for (int sweep = 0; sweep < 16; ++sweep) {
        const float off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        const float diag = A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2];
        if (off <= 1e-14f * diag || off == 0.0f) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            if (A[p][q] == 0.0f) continue;
            const float theta = (A[q][q] - A[p][p]) / (2.0f * A[p][q]);
            const float t = (theta >= 0.0f ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
            const float c = 1.0f / sqrtf(t * t + 1.0f), sn = t * c;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float akp = A[k][p], akq = A[k][q];
                A[k][p] = c * akp - sn * akq;
                A[k][q] = sn * akp + c * akq;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float apk = A[p][k], aqk = A[q][k];
                A[p][k] = c * apk - sn * aqk;
                A[q][k] = sn * apk + c * aqk;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float vkp = V[k][p], vkq = V[k][q];
                V[k][p] = c * vkp - sn * vkq;
                V[k][q] = sn * vkp + c * vkq;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

// Visit, 32 at a time, the particles of the sub-cells of the (2 rr + 1)^3 cells
// around the sample (cell c, fraction u) whose box lies closer than
// sqrt(reach2) cell widths; f(j, valid) per lane.  Row by row (z, y); a row's
// up to 40 sub-cells are tested by the lanes (two ballots) and the runs of
// reachable sub-cells are walked as contiguous sorted ranges.
template <typename F>
__device__ __forceinline__ void for_reach(const GridDev& g, const int c[3], const float u[3], int rr, float reach2,
                                          int lane, F&& f) {
    const int x0 = max(c[0] - rr, 0), x1 = min(c[0] + rr, g.dims[0] - 1);
    if (x0 > x1) return;
    const int nsubs = 8 * (x1 - x0 + 1);  // <= 40
    // squared x-distance of this lane's sub-cells k = lane and lane + 32 (cell x0 + k / 8, sub k % 8)
    float dx2[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int k = lane + 32 * h;
        const int cx = x0 + (k >> 3) - c[0];
        dx2[h] = slab_d2(u[0], (float)cx + 0.5f * (float)(k & 1));
    }
    for (int z = max(c[2] - rr, 0); z <= min(c[2] + rr, g.dims[2] - 1); ++z) {
        const float dz = (float)(z - c[2]);
        const float z0 = slab_d2(u[2], dz), z1 = slab_d2(u[2], dz + 0.5f);
        for (int y = max(c[1] - rr, 0); y <= min(c[1] + rr, g.dims[1] - 1); ++y) {
            const float dy = (float)(y - c[1]);
            const float y0 = slab_d2(u[1], dy), y1 = slab_d2(u[1], dy + 0.5f);
            const uint32_t row = ((uint32_t)z * (uint32_t)g.dims[1] + (uint32_t)y) * (uint32_t)g.dims[0];
            const uint32_t base = 8u * (row + (uint32_t)x0);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int k = lane + 32 * h;
                const int sb = k & 7;
                const float d2 = dx2[h] + ((sb & 2) ? y1 : y0) + ((sb & 4) ? z1 : z0);
                uint32_t m = __ballot_sync(kFull, k < nsubs && d2 < reach2);
                while (m) {
                    const int s0 = __ffs(m) - 1;
                    const uint32_t rest = ~(m >> s0);
                    const int len = rest ? __ffs(rest) - 1 : 32 - s0;  // length of the run of set bits at s0
                    m = (len + s0 >= 32) ? 0u : (m & ~(((1u << len) - 1u) << s0));
                    const uint32_t b = __ldg(g.sub + base + (uint32_t)(32 * h + s0));
                    const uint32_t e = __ldg(g.sub + base + (uint32_t)(32 * h + s0 + len));
                    for (uint32_t j0 = b; j0 < e; j0 += 32) {
                        const uint32_t j = j0 + (uint32_t)lane;
                        f(j, j < e);
                    }
                }
            }
        }
    }
}

// glm mat3 * vec3 (G[col][row]).
__device__ __forceinline__ void mat_vec(const float G[3][3], float x, float y, float z, float& ox, float& oy,
                                        float& oz) {
    ox = G[0][0] * x + G[1][0] * y + G[2][0] * z;
    oy = G[0][1] * x + G[1][1] * y + G[2][1] * z;
    oz = G[0][2] * x + G[1][2] * y + G[2][2] * z;
}

// WPCA and the anisotropic density at p (identical on every lane).  False when
// p has no particle within the extended radius (density 0).  The weighted
// moments are taken about p in one pass: mean = p + m, C = S / W - m m^T with
// m = sum w r / W and S = sum w r r^T, r = x - p (|r| < Hext, so no
// cancellation to speak of).  This march matches the reference to rounding,
// not bit for bit, so its sums use fused multiply-adds (__fmaf_rn; the file
// is compiled without contraction for the isotropic march's exact sums).
__device__ __forceinline__ bool aniso_eval(const GridDev& g, const AnisoDev& an, float px, float py, float pz, int lane,
                                           float G[3][3], float& detG, float& rho) {
    rho = 0.0f;
    Loc L;
    if (!locate(g, px, py, pz, L)) return false;
    float ws = 0.0f, mx = 0.0f, my = 0.0f, mz = 0.0f, cnt = 0.0f;
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c11 = 0.f, c12 = 0.f, c22 = 0.f;
    for_reach(g, L.c, L.u, 2, an.reach2_ext, lane, [&](uint32_t j, bool ok) {
        if (!ok) return;
        const float4 q = __ldg(g.pts + j);
        const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
        const float d2 = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx));
        if (d2 < an.hext2) {
            const float k = sqrtf(d2) * an.hext_inv;
            const float w = __fmaf_rn(-(k * k), k, 1.0f);
            ws += w;
            const float wx = w * rx, wy = w * ry, wz = w * rz;
            mx += wx;
            my += wy;
            mz += wz;
            c00 = __fmaf_rn(wx, rx, c00);
            c01 = __fmaf_rn(wx, ry, c01);
            c02 = __fmaf_rn(wx, rz, c02);
            c11 = __fmaf_rn(wy, ry, c11);
            c12 = __fmaf_rn(wy, rz, c12);
            c22 = __fmaf_rn(wz, rz, c22);
            cnt += 1.0f;
        }
    });
    ws = warp_sum(ws);
    cnt = warp_sum(cnt);
    if (cnt == 0.0f) return false;
    const float iw = 1.0f / ws;
    const float m0 = warp_sum(mx) * iw, m1 = warp_sum(my) * iw, m2 = warp_sum(mz) * iw;
    float A[3][3];
    A[0][0] = warp_sum(c00) * iw - m0 * m0;
    A[0][1] = A[1][0] = warp_sum(c01) * iw - m0 * m1;
    A[0][2] = A[2][0] = warp_sum(c02) * iw - m0 * m2;
    A[1][1] = warp_sum(c11) * iw - m1 * m1;
    A[1][2] = A[2][1] = warp_sum(c12) * iw - m1 * m2;
    A[2][2] = warp_sum(c22) * iw - m2 * m2;
    float sg[3], R[3][3];
    eig3_jacobi(A, sg, R);
    float S[3];
    if ((int)fminf(cnt, 8192.0f) <= an.n_eps) {
        S[0] = S[1] = S[2] = an.k_n;
    } else {
        const float mxs = fmaxf(sg[0], fmaxf(sg[1], sg[2]));
        const float mn = mxs / an.k_r;
#pragma unroll
        for (int k = 0; k < 3; ++k) S[k] = fmaxf(sg[k], mn) * an.k_s;
    }
    const float is[3] = {1.0f / S[0], 1.0f / S[1], 1.0f / S[2]};
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            G[cc][r] = an.hinv * ((R[r][0] * R[cc][0]) * is[0] + (R[r][1] * R[cc][1]) * is[1] +
                                  (R[r][2] * R[cc][2]) * is[2]);
    detG = G[0][0] * (G[1][1] * G[2][2] - G[2][1] * G[1][2]) - G[1][0] * (G[0][1] * G[2][2] - G[2][1] * G[0][2]) +
           G[2][0] * (G[0][1] * G[1][2] - G[1][1] * G[0][2]);
    // anisotropic density over the particles within H (AnisotropicKernel::W)
    const float sd = an.sig * detG;
    float sum = 0.0f;
    for_reach(g, L.c, L.u, 1, an.reach2, lane, [&](uint32_t j, bool ok) {
        if (!ok) return;
        const float4 q = __ldg(g.pts + j);
        const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
        if (__fmaf_rn(rz, rz, __fmaf_rn(ry, ry, rx * rx)) >= an.h2) return;
        const float gx = __fmaf_rn(G[2][0], rz, __fmaf_rn(G[1][0], ry, G[0][0] * rx));
        const float gy = __fmaf_rn(G[2][1], rz, __fmaf_rn(G[1][1], ry, G[0][1] * rx));
        const float gz = __fmaf_rn(G[2][2], rz, __fmaf_rn(G[1][2], ry, G[0][2] * rx));
        float qq = __fmaf_rn(gz, gz, __fmaf_rn(gy, gy, gx * gx));
        if (qq >= an.h2) return;
        qq = sqrtf(qq) * an.hinv;
        if (qq >= 0.5f) {
            const float q_ = 1.0f - qq;
            sum = __fmaf_rn(sd, 2.0f * q_ * q_ * q_, sum);
        } else {
            sum = __fmaf_rn(sd, __fmaf_rn(6.0f, qq * qq * qq - qq * qq, 1.0f), sum);
        }
    });
    rho = warp_sum(sum);
    return true;
}

// Sum of AnisotropicKernel::gradW at p with the G of p (identical on every lane).
__device__ __forceinline__ void aniso_grad(const GridDev& g, const AnisoDev& an, float px, float py, float pz, int lane,
                                           const float G[3][3], float detG, float& ox, float& oy, float& oz) {
    float sx = 0.f, sy = 0.f, sz = 0.f;
    Loc L;
    if (locate(g, px, py, pz, L)) {
        for_reach(g, L.c, L.u, 1, an.reach2, lane, [&](uint32_t j, bool ok) {
            if (!ok) return;
            const float4 q = __ldg(g.pts + j);
            const float rx = q.x - px, ry = q.y - py, rz = q.z - pz;
            if (dot3(rx, ry, rz, rx, ry, rz) >= an.h2) return;
            float gx, gy, gz;
            mat_vec(G, rx, ry, rz, gx, gy, gz);
            const float rn = dot3(gx, gy, gz, gx, gy, gz);
            if (rn >= an.h2 || rn == 0.0f) return;
            const float rl = sqrtf(rn);
            const float qq = rl * an.hinv;
            const float inv = 1.0f / sqrtf(rn);
            const float den = rl * an.h;
            const float nx = (gx * inv) / den, ny = (gy * inv) / den, nz = (gz * inv) / den;
            if (qq >= 0.5f) {
                const float q_ = 1.0f - qq;
                const float a0 = -an.sig * detG;
                sx += (a0 * nx) * (6.0f * q_ * q_);
                sy += (a0 * ny) * (6.0f * q_ * q_);
                sz += (a0 * nz) * (6.0f * q_ * q_);
            } else {
                const float f = 6.0f * (3.0f * qq * qq - 2.0f * qq);
                const float a0 = an.sig * detG;
                sx += (a0 * nx) * f;
                sy += (a0 * ny) * f;
                sz += (a0 * nz) * f;
            }
        });
    }
    ox = warp_sum(sx);
    oy = warp_sum(sy);
    oz = warp_sum(sz);
}

struct AnisoCount {
    uint64_t evals = 0, hits = 0, rays = 0, started = 0, skipped = 0;
};

// One started ray (pixel idx) of view `a`, marched with the whole warp.
template <bool STATS>
__device__ __forceinline__ void aniso_ray(const MarchArgs& a, const AnisoDev& an, uint64_t idx, int lane,
                                          AnisoCount& c) {
    const int px = (int)(idx % (uint64_t)a.W), py = (int)(idx / (uint64_t)a.W);
    float p[3], s[3];
    ray_setup(a, px, py, a.zbuf[idx], p, s);
    float q[3] = {p[0], p[1], p[2]};
    float G[3][3], detG = 0.0f, rho = 0.0f;
    bool hit = false;
    for (int i = 0; i < a.max_steps; ++i) {
        p[0] = p[0] + s[0];
        p[1] = p[1] + s[1];
        p[2] = p[2] + s[2];
        if (a.skip_mode == FM_SKIP_REFERENCE) ref_skip(a.g, p[0], p[1], p[2], s[0], s[1], s[2], a.status);
        if (outside_forever(a.g, p[0], p[1], p[2], s[0], s[1], s[2])) break;
        if (a.iso > 0.0f && zero_density(a.g, p[0], p[1], p[2])) {
            // no particle within the support radius: the anisotropic density (its
            // terms need |r| < H) is exactly 0, below iso; leaving the box for good ends the ray
            if (leaving_zero_box(a.g, p[0], p[1], p[2], s[0], s[1], s[2])) break;
            if (STATS) c.skipped++;
            q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
            continue;
        }
        if (a.skip_mode == FM_SKIP_EXACT && a.iso > 0.0f) {
            // no particle within the support radius of the sample's bound box:
            // the anisotropic density is exactly 0
            Loc L;
            if (locate(a.g, p[0], p[1], p[2], L) && box_bound(a.g, L) == 0.0f) {
                if (STATS) c.skipped++;
                q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
                continue;
            }
        }
        if (STATS) c.evals++;
        aniso_eval(a.g, an, p[0], p[1], p[2], lane, G, detG, rho);
        if (rho >= a.iso) {
            hit = true;
            break;
        }
        q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
    }
    float n0 = 0.f, n1 = 0.f, n2 = 0.f;
    if (hit) {
        for (int b = 0; b < a.bisect; ++b) {
            const float m[3] = {(q[0] + p[0]) * 0.5f, (q[1] + p[1]) * 0.5f, (q[2] + p[2]) * 0.5f};
            if (STATS) c.evals++;
            aniso_eval(a.g, an, m[0], m[1], m[2], lane, G, detG, rho);
            if (rho >= a.iso) { p[0] = m[0]; p[1] = m[1]; p[2] = m[2]; }
            else { q[0] = m[0]; q[1] = m[1]; q[2] = m[2]; }
        }
        // RayMarcher.cpp:411-416: the gradient sum with the G of the hit point
        if (STATS) c.evals++;
        aniso_eval(a.g, an, p[0], p[1], p[2], lane, G, detG, rho);
        float gx, gy, gz;
        aniso_grad(a.g, an, p[0], p[1], p[2], lane, G, detG, gx, gy, gz);
        const float gi = 1.0f / sqrtf(dot3(gx, gy, gz, gx, gy, gz));
        n0 = gx * gi;
        n1 = gy * gi;
        n2 = gz * gi;
        if (STATS) c.hits++;
    }
    if (lane == 0) write_pixel(a, idx, px, py, hit, p[0], p[1], p[2], n0, n1, n2);
}

// One chunk of 32 consecutive pixels of view `a` (from pixel `base`): the
// started rays among them are marched one after the other with the whole warp.
template <bool STATS>
__device__ __forceinline__ void aniso_chunk(const MarchArgs& a, const AnisoDev& an, uint64_t base, int lane,
                                            AnisoCount& c) {
    const uint64_t npx = (uint64_t)a.W * (uint64_t)a.Hh;
    const uint64_t my = base + (uint64_t)lane;
    const bool valid = my < npx;
    const float zl = valid ? a.zbuf[my] : 1.0f;
    uint32_t todo = __ballot_sync(kFull, valid && zl != 1.0f);
    if (STATS) { c.rays += valid; c.started += valid && zl != 1.0f; }
    // misses without a ray start are written by their own lane
    if (valid && zl == 1.0f)
        write_pixel(a, my, (int)(my % (uint64_t)a.W), (int)(my / (uint64_t)a.W), false, 0.f, 0.f, 0.f, 0.f, 0.f,
                    0.f);
    while (todo) {
        const int src = __ffs(todo) - 1;
        todo &= todo - 1u;
        aniso_ray<STATS>(a, an, base + (uint64_t)src, lane, c);
    }
}

// Single view: the started pixels into a list (in any order) for k_march_aniso
// to take one ray at a time, so the launch does not end on a chunk of many long
// rays; pixels without a ray start get their miss outputs here.
template <bool STATS>
__global__ void k_aniso_starts(const MarchArgs a, uint32_t* __restrict__ list, unsigned int* __restrict__ n_list) {
    const uint64_t npx = (uint64_t)a.W * (uint64_t)a.Hh;
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const bool valid = i < npx;
    const bool started = valid && a.zbuf[i] != 1.0f;
    const uint32_t m = __ballot_sync(kFull, started);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(n_list, (unsigned)__popc(m));
    base = __shfl_sync(kFull, base, 0);
    if (started) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
    else if (valid) write_pixel(a, i, (int)(i % (uint64_t)a.W), (int)(i / (uint64_t)a.W), false, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
    if (STATS) {
        const uint32_t v = __ballot_sync(kFull, valid);
        if (lane == 0 && v) atomicAdd(a.stats + 0, (unsigned long long)__popc(v));
        if (lane == 0 && m) atomicAdd(a.stats + 1, (unsigned long long)__popc(m));
    }
}

// Persistent warps take chunks of 32 consecutive pixels from a counter.
// BATCH: chunk t belongs to view find_view(pfx, t) of `views` / `aviews`
// (views without anisotropic rays own no chunks); otherwise to view `a`.
// Single view (list != null): warps take one started ray at a time from the
// list k_aniso_starts wrote.
template <bool STATS, bool BATCH>
__global__ void __launch_bounds__(kThreads)
    k_march_aniso(const __grid_constant__ MarchArgs a, const __grid_constant__ AnisoDev an,
                  const MarchArgs* __restrict__ views, const AnisoDev* __restrict__ aviews,
                  const uint32_t* __restrict__ pfx, int nviews, uint32_t nchunks, const uint32_t* __restrict__ list,
                  const unsigned int* __restrict__ n_list) {
    const int lane = threadIdx.x & 31;
    AnisoCount c;
    const unsigned nl = BATCH ? 0u : *n_list;
    for (;;) {
        unsigned k = 0;
        if (lane == 0) k = atomicAdd(a.tile_counter, 1u);
        k = __shfl_sync(kFull, k, 0);
        if constexpr (BATCH) {
            if (k >= nchunks) break;
            const int v = find_view(pfx, nviews, k);
            aniso_chunk<STATS>(views[v], aviews[v], (uint64_t)(k - __ldg(pfx + v)) * 32u, lane, c);
        } else {
            if (k >= nl) break;
            aniso_ray<STATS>(a, an, (uint64_t)__ldg(list + k), lane, c);
        }
    }
    if (STATS) {
        // fm_march_stats order: rays, started, hits, evals, candidates, skipped
        const unsigned long long v[6] = {c.rays, c.started, lane == 0 ? c.hits : 0ull, lane == 0 ? c.evals : 0ull,
                                         0ull, lane == 0 ? c.skipped : 0ull};
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            unsigned long long x = v[j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
            if (lane == 0 && x) atomicAdd(a.stats + j, x);
        }
    }
}

AnisoDev make_aniso(const fm_scene* s, const fm_aniso_params* ap) {
    AnisoDev an;
    an.hext = ap->radius_mult * s->support;  // Dataset.cpp:175
    {
        const float r = ap->radius_mult * (1.0f + 1.0e-3f), r1 = 1.0f + 1.0e-3f;
        an.reach2_ext = r * r;
        an.reach2 = r1 * r1;
    }
    an.hext2 = an.hext * an.hext;
    an.hext_inv = 1.0f / an.hext;
    an.h = s->support;
    an.h2 = s->support * s->support;
    an.hinv = 1.0f / s->support;
    an.sig = 8.0f / 3.14159265358979323846f;
    an.k_n = ap->k_n;
    an.k_r = ap->k_r;
    an.k_s = ap->k_s;
    an.n_eps = ap->n_eps;
    return an;
}

template <bool STATS, bool BATCH>
int launch_aniso_variant(fm_ctx* ctx, const MarchArgs& a, const AnisoDev& an, const MarchArgs* views,
                         const AnisoDev* aviews, const uint32_t* pfx, int nviews, uint32_t nchunks, uint32_t* list,
                         unsigned int* n_list, cudaStream_t st) {
    if (!BATCH) {
        const uint64_t npx = (uint64_t)a.W * (uint64_t)a.Hh;
        k_aniso_starts<STATS><<<(unsigned)((npx + 255) / 256), 256, 0, st>>>(a, list, n_list);
        FM_CUDA(ctx, cudaGetLastError());
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_march_aniso<STATS, BATCH>, kThreads, 0);
    if (per_sm < 1) per_sm = 1;
    const unsigned blocks = (unsigned)(ctx->sm_count * per_sm);
    k_march_aniso<STATS, BATCH><<<blocks, kThreads, 0, st>>>(a, an, views, aviews, pfx, nviews, nchunks, list, n_list);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace

size_t aniso_view_bytes() { return sizeof(AnisoDev); }

void aniso_view(const fm_scene* s, const fm_aniso_params* ap, void* out) {
    const AnisoDev an = make_aniso(s, ap);
    std::memcpy(out, &an, sizeof(an));
}

int launch_march_aniso_batch(fm_ctx* ctx, const MarchArgs& a, const MarchArgs* d_views, const void* d_aviews,
                             const uint32_t* d_pfx, int nviews, uint32_t nchunks, cudaStream_t st) {
    if (nchunks == 0) return FM_OK;
    AnisoDev none;
    std::memset(&none, 0, sizeof(none));
    if (a.stats)
        return launch_aniso_variant<true, true>(ctx, a, none, d_views, (const AnisoDev*)d_aviews, d_pfx, nviews,
                                                nchunks, nullptr, nullptr, st);
    return launch_aniso_variant<false, true>(ctx, a, none, d_views, (const AnisoDev*)d_aviews, d_pfx, nviews, nchunks,
                                             nullptr, nullptr, st);
}

int launch_march_aniso(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p,
                       const fm_aniso_params* ap, const MarchOutDev& o, cudaStream_t st) {
    MarchArgs a = march_view_args(s, cam, p, o, ctx->tile);
    a.stats = ctx->stats_enabled ? ctx->d_stats : nullptr;
    a.status = ctx->d_status;
    unsigned int* slot = ctx->d_work + (ctx->work_slot++ % kWorkSlots) * 32;
    a.tile_counter = slot;
    FM_CUDA(ctx, cudaMemsetAsync(slot, 0, 2 * sizeof(unsigned int), st));
    const uint64_t npx = (uint64_t)cam->width * (uint64_t)cam->height;
    if (ctx->aniso_list.bytes < npx * 4) {
        FM_CUDA(ctx, cudaStreamSynchronize(st));  // the list may be in use by an earlier launch
        if (!grow_buf(ctx->aniso_list, npx * 4)) return set_err(ctx, FM_ERR_OOM, "ray list allocation failed");
    }
    uint32_t* list = (uint32_t*)ctx->aniso_list.p;
    const AnisoDev an = make_aniso(s, ap);
    if (a.stats) return launch_aniso_variant<true, false>(ctx, a, an, nullptr, nullptr, nullptr, 0, 0, list, slot + 1, st);
    return launch_aniso_variant<false, false>(ctx, a, an, nullptr, nullptr, nullptr, 0, 0, list, slot + 1, st);
}

int launch_density(fm_ctx* ctx, const fm_scene* s, const float* d_xyz, uint64_t n, uint32_t stride, float* d_out,
                   cudaStream_t st) {
    if (n == 0) return FM_OK;
    k_density_probe<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(grid_dev(s), make_kernel(s->support), d_xyz, n,
                                                                 stride, d_out);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

int launch_march(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p,
                 const MarchOutDev& o, cudaStream_t st, DevBuf* queue) {
    MarchArgs a = march_view_args(s, cam, p, o, ctx->tile);
    a.stats = ctx->stats_enabled ? ctx->d_stats : nullptr;
    a.status = ctx->d_status;
    // fresh counters per launch (a ring of slots, so launches on different
    // streams do not share them): tiles, queue tail, queue head, second-pass
    // groups, second queue tail and head
    unsigned int* slot = ctx->d_work + (ctx->work_slot++ % kWorkSlots) * 32;
    a.tile_counter = slot;
    a.q_tail = slot + 1;
    a.q_head = slot + 2;
    a.grp_counter = slot + 3;
    a.q2_tail = slot + 4;
    a.q2_head = slot + 5;
    FM_CUDA(ctx, cudaMemsetAsync(slot, 0, 6 * sizeof(unsigned int), st));
    const uint64_t entries = long_queue_entries((uint64_t)cam->width * (uint64_t)cam->height, ctx->tile.qlimit);
    const bool regroup = ctx->tile.cap2 > 0 && !queue;
    DevBuf& longq = queue ? *queue : ctx->longq;
    const uint64_t nkeys = (uint64_t)a.ntiles + 1;
    const bool small = longq.bytes < entries * 64 ||
                       (regroup && (ctx->longq2.bytes < entries * 64 || ctx->rg_order.bytes < entries * 4 ||
                                    ctx->rg_keys.bytes < nkeys * 4 || ctx->rg_tmp.bytes < scan_words(nkeys) * 4));
    if (small) {
        FM_CUDA(ctx, cudaStreamSynchronize(st));  // the buffers may be in use by an earlier launch
        if (!grow_buf(longq, entries * 64) ||
            (regroup && (!grow_buf(ctx->longq2, entries * 64) || !grow_buf(ctx->rg_order, entries * 4) ||
                         !grow_buf(ctx->rg_keys, nkeys * 4) || !grow_buf(ctx->rg_tmp, scan_words(nkeys) * 4))))
            return set_err(ctx, FM_ERR_OOM, "long-ray queue allocation failed");
    }
    a.longq = (float4*)longq.p;
    a.q_cap = (unsigned int)entries;
    if (regroup) {
        a.longq2 = (float4*)ctx->longq2.p;
        a.order = (uint32_t*)ctx->rg_order.p;
        a.keys = (uint32_t*)ctx->rg_keys.p;
        a.scan_tmp = (uint32_t*)ctx->rg_tmp.p;
    }
    return launch_march_kernels(ctx, a, nullptr, nullptr, 0, st);
}

}  // namespace fm
