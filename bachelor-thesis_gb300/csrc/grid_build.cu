// grid_build.cu -- GPU uniform-grid build of a particle frame.
//
// Replaces Frame::BuildSearch / ComputeAABB / BuildDensityGrid
// (src/app/Dataset.cpp:49-165) and the cell table inside the CompactNSearch
// library the reference calls.  Integer results are bit-identical to the
// reference formulas:
//   AABB            min/max over all particles, padded by the support radius
//                   (Dataset.cpp:78-92); min/max is exact, the padding is one
//                   FP32 add/sub done on the host exactly as the reference does.
//   dims            ceil((max - min) / cell) (Dataset.cpp:102-104).
//   cell index      floor((p - min) * (1/cell)), x + y*W + z*W*H
//                   (QueryDensityGrid, Dataset.cpp:28-40).
//   order           stable counting sort by key = cell * 8 + sub-cell, where
//                   the sub-cell splits each cell into 2x2x2 half-width slabs
//                   (sx = frac(f) >= 0.5, sub = sx + 2 sy + 4 sz); an LSD radix
//                   sort of the key, 8 bits per pass, input index as the
//                   value, so particles of a sub-cell keep their input order.
//   tables          sub[k] = exclusive prefix sum of the key counts
//                   (8 * n_cells + 1 entries); cell c spans [sub[8c], sub[8c+8]).
// Data layout in HBM: float4 sorted positions (16 B, one 128-bit load per
// particle), the uint32 sub-cell start table, uint32 cell and sorted->input
// index arrays.  The march reads whole cell rows as contiguous ranges and
// skips sub-cells out of reach of a sample.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fm_internal.cuh"

namespace fm {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / kWarp;

__device__ __forceinline__ uint32_t f2ord(float f) {
    uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__host__ __device__ inline float ord2f(uint32_t k) {
    uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// mm[0..2] = ordered min, mm[3..5] = ordered max, mm[6] = count of non-finite coordinates.
__global__ void k_aabb(const float* __restrict__ xyz, uint64_t n, uint32_t stride, uint32_t* __restrict__ mm) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t bad = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float* p = xyz + i * stride;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float v = p[a];
            if (!isfinite(v)) { bad++; continue; }
            mn[a] = fminf(mn[a], v);
            mx[a] = fmaxf(mx[a], v);
        }
    }
    __shared__ uint32_t s[7][32];
    uint32_t k[7];
#pragma unroll
    for (int a = 0; a < 3; ++a) { k[a] = f2ord(mn[a]); k[3 + a] = f2ord(mx[a]); }
    k[6] = bad;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            k[a] = min(k[a], __shfl_xor_sync(0xffffffffu, k[a], o));
            k[3 + a] = max(k[3 + a], __shfl_xor_sync(0xffffffffu, k[3 + a], o));
        }
        k[6] += __shfl_xor_sync(0xffffffffu, k[6], o);
    }
    int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
    if (l == 0)
        for (int a = 0; a < 7; ++a) s[a][w] = k[a];
    __syncthreads();
    if (threadIdx.x == 0) {
        int nw = blockDim.x / kWarp;
        for (int j = 1; j < nw; ++j) {
            for (int a = 0; a < 3; ++a) {
                k[a] = min(k[a], s[a][j]);
                k[3 + a] = max(k[3 + a], s[3 + a][j]);
            }
            k[6] += s[6][j];
        }
        for (int a = 0; a < 3; ++a) {
            atomicMin(&mm[a], k[a]);
            atomicMax(&mm[3 + a], k[3 + a]);
        }
        if (k[6]) atomicAdd(&mm[6], k[6]);
    }
}

struct GridParams {
    float min[3];
    float inv;
    int dims[3];
};

// Per-particle cell (QueryDensityGrid formula; coordinates clamped into the
// grid, which the support-radius padding guarantees for finite input), the
// sort key cell * 8 + sub-cell, and the key histogram.
__device__ __forceinline__ uint32_t cell_key(const float* p, const GridParams& g, uint32_t& lin) {
    int c[3];
    uint32_t sub = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float f = (p[a] - g.min[a]) * g.inv;
        int v = (int)floorf(f);
        c[a] = min(max(v, 0), g.dims[a] - 1);
        if (f - (float)c[a] >= 0.5f) sub |= 1u << a;
    }
    lin = (uint32_t)c[0] + (uint32_t)c[1] * (uint32_t)g.dims[0] +
          (uint32_t)c[2] * (uint32_t)g.dims[0] * (uint32_t)g.dims[1];
    return lin * 8u + sub;
}

__global__ void k_cells(const float* __restrict__ xyz, uint64_t n, uint32_t stride, GridParams g,
                        uint32_t* __restrict__ cell, uint32_t* __restrict__ key, uint32_t* __restrict__ count) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t lin;
    const uint32_t k = cell_key(xyz + i * stride, g, lin);
    cell[i] = lin;
    key[i] = k;
    atomicAdd(&count[k], 1u);
}

// ---- single-sync build: grid parameters computed on the device ------------
// The bounds pass accumulates the AABB into the bounds words; a one-thread
// pass turns those into the grid (the reference's FP32 order,
// Dataset.cpp:89-104: max + pad, min - pad, ceil(extent / cell), 1 / cell;
// device division and ceil are IEEE-exact like the host's), checks it against
// the cell capacity the host launched the rest of the build for and writes a
// record.  Every later pass reads the record (through L1: one line that all
// threads read) and does nothing unless status is kGridOk; the host reads it
// once, after the build.
enum : uint32_t { kGridOk = 0, kGridNonFinite = 1, kGridExtent = 2, kGridTooMany = 3, kGridOverCapacity = 4 };

struct GridInfo {
    GridParams g;
    uint32_t status;
    float max[3];
    uint32_t ncells;
    uint32_t n_long;  // segments longer than kShortSeg, listed by k_segsort_gather
};

// Bounds words: [0..2] ordered min, [3..5] ordered max, [6] non-finite
// coordinates.  Between builds they hold (~0, ~0, ~0, 0, 0, 0, 0): the record
// pass puts them back once it has read them.
constexpr int kBoundsThreads = 256;

__device__ void reset_bounds(uint32_t* mm) {
    for (int a = 0; a < 3; ++a) {
        mm[a] = 0xffffffffu;
        mm[3 + a] = 0u;
    }
    mm[6] = 0u;
}

__device__ GridInfo grid_from_bounds(const uint32_t* mm, float support, uint64_t capacity) {
    uint32_t h[7];
    for (int a = 0; a < 7; ++a) h[a] = mm[a];
    GridInfo gi;
    gi.status = h[6] ? kGridNonFinite : kGridOk;
    gi.n_long = 0;
    gi.ncells = 0;
    const float pad = 1.0f * support, cell = 1.0f * support;
    uint64_t ncells = 1;
    for (int a = 0; a < 3; ++a) {
        const float lo = ord2f(h[a]), hi = ord2f(h[3 + a]);
        gi.max[a] = hi + pad;
        gi.g.min[a] = lo - pad;
        const float ext = gi.max[a] - gi.g.min[a];
        const float d = ceilf(ext / cell);
        if (!(d >= 1.0f && d < 1.0e6f)) {
            if (gi.status == kGridOk) gi.status = kGridExtent;
            gi.g.dims[a] = 1;
        } else {
            gi.g.dims[a] = (int)d;
        }
        ncells *= (uint64_t)gi.g.dims[a];
    }
    gi.g.inv = 1.0f / cell;
    if (gi.status == kGridOk) {
        if (ncells > (1ull << 28)) {
            gi.status = kGridTooMany;
        } else {
            gi.ncells = (uint32_t)ncells;
            if (ncells > capacity) gi.status = kGridOverCapacity;
        }
    }
    return gi;
}

// Bounds pass over positions with a stride of 3 floats at a 16-byte aligned
// base (VEC3: the 3n floats read as float4; component c of float4 q holds
// axis (q + c) % 3, and the grid stride is a multiple of 3 float4s, so all of
// a thread's float4s share q % 3 and the axes are rotated into place once at
// the end) or any stride (one float per load).
template <bool VEC3>
__global__ void __launch_bounds__(kBoundsThreads)
    k_grid_bounds(const float* __restrict__ xyz, uint64_t n, uint32_t stride, uint32_t* __restrict__ mm) {
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t bad = 0;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, step = (uint64_t)gridDim.x * blockDim.x;
    if (VEC3) {
        const uint64_t nf = 3 * n, nq = nf / 4;
        float smn[3] = {INFINITY, INFINITY, INFINITY}, smx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint64_t q = t0; q < nq; q += step) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(xyz) + q);
            const float c[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int sl = j == 3 ? 0 : j;
                if (!isfinite(c[j])) { bad++; continue; }
                smn[sl] = fminf(smn[sl], c[j]);
                smx[sl] = fmaxf(smx[sl], c[j]);
            }
        }
        const uint32_t r = (uint32_t)(t0 % 3);
#pragma unroll
        for (int sl = 0; sl < 3; ++sl) {
            const uint32_t a = (r + (uint32_t)sl) % 3u;
            // axis a, unrolled into selects (no indexed register arrays)
            mn[0] = a == 0 ? smn[sl] : mn[0]; mx[0] = a == 0 ? smx[sl] : mx[0];
            mn[1] = a == 1 ? smn[sl] : mn[1]; mx[1] = a == 1 ? smx[sl] : mx[1];
            mn[2] = a == 2 ? smn[sl] : mn[2]; mx[2] = a == 2 ? smx[sl] : mx[2];
        }
        for (uint64_t j = 4 * nq + t0; j < nf; j += step) {  // the last nf % 4 floats
            const float v = xyz[j];
            const uint32_t a = (uint32_t)(j % 3);
            if (!isfinite(v)) { bad++; continue; }
            if (a == 0) { mn[0] = fminf(mn[0], v); mx[0] = fmaxf(mx[0], v); }
            if (a == 1) { mn[1] = fminf(mn[1], v); mx[1] = fmaxf(mx[1], v); }
            if (a == 2) { mn[2] = fminf(mn[2], v); mx[2] = fmaxf(mx[2], v); }
        }
    } else {
        for (uint64_t i = t0; i < n; i += step) {
            const float* p = xyz + i * stride;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float v = p[a];
                if (!isfinite(v)) { bad++; continue; }
                mn[a] = fminf(mn[a], v);
                mx[a] = fmaxf(mx[a], v);
            }
        }
    }
    __shared__ uint32_t s[7][kBoundsThreads / kWarp];
    uint32_t k[7];
#pragma unroll
    for (int a = 0; a < 3; ++a) { k[a] = f2ord(mn[a]); k[3 + a] = f2ord(mx[a]); }
    k[6] = bad;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            k[a] = min(k[a], __shfl_xor_sync(0xffffffffu, k[a], o));
            k[3 + a] = max(k[3 + a], __shfl_xor_sync(0xffffffffu, k[3 + a], o));
        }
        k[6] += __shfl_xor_sync(0xffffffffu, k[6], o);
    }
    const int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
    if (l == 0)
        for (int a = 0; a < 7; ++a) s[a][w] = k[a];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 1; j < kBoundsThreads / kWarp; ++j) {
            for (int a = 0; a < 3; ++a) {
                k[a] = min(k[a], s[a][j]);
                k[3 + a] = max(k[3 + a], s[3 + a][j]);
            }
            k[6] += s[6][j];
        }
        for (int a = 0; a < 3; ++a) {
            atomicMin(&mm[a], k[a]);
            atomicMax(&mm[3 + a], k[3 + a]);
        }
        if (k[6]) atomicAdd(&mm[6], k[6]);
    }
}

__global__ void k_grid_record(uint32_t* __restrict__ mm, float support, uint64_t capacity,
                              GridInfo* __restrict__ info) {
    *info = grid_from_bounds(mm, support, capacity);
    reset_bounds(mm);
}

// Cell pass: per particle the cell, the key and its rank among the particles
// of its key (the histogram's atomic returns it; the order of equal keys is
// arbitrary here and fixed by the segment sort).
__global__ void k_cells_info(const float* __restrict__ xyz, uint64_t n, uint32_t stride,
                             const GridInfo* __restrict__ info, uint32_t* __restrict__ cell,
                             uint32_t* __restrict__ key, uint32_t* __restrict__ rank, uint32_t* __restrict__ count) {
    if (info->status != kGridOk) return;
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GridParams g = info->g;
    uint32_t lin;
    const uint32_t k = cell_key(xyz + i * stride, g, lin);
    cell[i] = lin;
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1u);
}

// ---- exclusive scan (uint32), multi-level ---------------------------------
// in and out may alias (in-place scan): each thread reads its items before any write.
__global__ void k_scan_tile(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t s_warp[kScanThreads / kWarp];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        v[j] = (base + j < n) ? in[base + j] : 0u;
        sum += v[j];
    }
    int l = threadIdx.x % kWarp, w = threadIdx.x / kWarp;
    uint32_t inc = sum;
#pragma unroll
    for (int o = 1; o < kWarp; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (l >= o) inc += t;
    }
    if (l == kWarp - 1) s_warp[w] = inc;
    __syncthreads();
    if (w == 0) {
        uint32_t x = s_warp[l];
#pragma unroll
        for (int o = 1; o < kWarp; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
            if (l >= o) x += t;
        }
        s_warp[l] = x;  // inclusive over warps
    }
    __syncthreads();
    uint32_t run = (inc - sum) + (w > 0 ? s_warp[w - 1] : 0u);
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == kScanThreads - 1 && tile_sums) tile_sums[blockIdx.x] = s_warp[kScanThreads / kWarp - 1];
}

__global__ void k_scan_add(uint32_t* __restrict__ out, uint64_t n, const uint32_t* __restrict__ tile_offsets) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] += tile_offsets[i / kScanTile];
}

// Second pass of a two-launch scan: the block adds the sum of all earlier
// tiles' totals (read from tile_sums and reduced by the block itself: at most
// kScanDirectTiles of them) to its 256 items, all inside one tile.
constexpr uint64_t kScanDirectTiles = 2048;
constexpr int kScanAddThreads = 256;
static_assert(kScanTile % kScanAddThreads == 0, "an add block stays inside one tile");

__global__ void __launch_bounds__(kScanAddThreads)
    k_scan_add_sums(uint32_t* __restrict__ out, uint64_t n, const uint32_t* __restrict__ tile_sums) {
    __shared__ uint32_t s_part[kScanAddThreads / kWarp];
    const uint64_t i0 = (uint64_t)blockIdx.x * kScanAddThreads;
    const uint32_t tile = (uint32_t)(i0 / kScanTile);
    uint32_t part = 0;
    for (uint32_t j = threadIdx.x; j < tile; j += kScanAddThreads) part += tile_sums[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    const int w = threadIdx.x / kWarp, l = threadIdx.x % kWarp;
    if (l == 0) s_part[w] = part;
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (int j = 0; j < kScanAddThreads / kWarp; ++j) off += s_part[j];
    const uint64_t i = i0 + threadIdx.x;
    if (i < n) out[i] += off;
}

// Words of temporary storage exclusive_scan needs for n items.
uint64_t scan_tmp_words(uint64_t n) {
    uint64_t w = 0;
    while (n > (uint64_t)kScanTile) {
        n = (n + kScanTile - 1) / kScanTile;
        w += 2 * n + 64;
    }
    return w + 64;
}

// out[i] = sum_{j<i} in[j]; in may equal out.
void exclusive_scan(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, cudaStream_t st) {
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles <= 1) {
        k_scan_tile<<<1, kScanThreads, 0, st>>>(in, out, n, nullptr);
        return;
    }
    uint32_t* sums = tmp;
    uint32_t* offs = tmp + tiles + 32;
    k_scan_tile<<<(unsigned)tiles, kScanThreads, 0, st>>>(in, out, n, sums);
    if (tiles <= kScanDirectTiles) {
        k_scan_add_sums<<<(unsigned)((n + kScanAddThreads - 1) / kScanAddThreads), kScanAddThreads, 0, st>>>(out, n,
                                                                                                            sums);
        return;
    }
    exclusive_scan(sums, offs, tiles, offs + tiles + 32, st);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, offs);
}

// ---- stable LSD radix sort pass (8-bit digit) -----------------------------
__global__ void k_radix_hist(const uint32_t* __restrict__ keys, uint64_t n, int shift, uint32_t nblocks,
                             uint32_t* __restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int it = 0; it < kSortItems; ++it) {
        uint64_t e = base + (uint64_t)it * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(uint64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Scatter one digit pass.  Elements keep their order within a digit: a tile
// is walked in rounds of 256 consecutive elements, ranks inside a round come
// from warp match masks plus per-warp digit counts, and blocks are ordered by
// the digit-major scanned histogram.  vals_in == nullptr: the value is the
// element index (first pass).
__global__ void k_radix_scatter(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
                                uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint64_t n,
                                int shift, uint32_t nblocks, const uint32_t* __restrict__ offs) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_tot[256];
    __shared__ uint32_t s_w[kSortWarps][256];
    const int t = threadIdx.x, l = t % kWarp, w = t / kWarp;
    s_base[t] = offs[(uint64_t)t * nblocks + blockIdx.x];
#pragma unroll
    for (int j = 0; j < kSortWarps; ++j) s_w[j][t] = 0;
    __syncthreads();
    const uint32_t lt = (1u << l) - 1u;
    uint64_t base = (uint64_t)blockIdx.x * kSortTile;
    for (int it = 0; it < kSortItems; ++it) {
        uint64_t e = base + (uint64_t)it * kSortThreads + t;
        bool valid = e < n;
        uint32_t key = valid ? keys_in[e] : 0u;
        uint32_t val = valid ? (vals_in ? vals_in[e] : (uint32_t)e) : 0u;
        uint32_t d = valid ? ((key >> shift) & 255u) : (0x10000u + l);
        uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t rank = __popc(peers & lt);
        if (valid && rank == 0) s_w[w][d] = __popc(peers);
        __syncthreads();
        {
            uint32_t run = 0;
#pragma unroll
            for (int j = 0; j < kSortWarps; ++j) {
                uint32_t c = s_w[j][t];
                s_w[j][t] = run;
                run += c;
            }
            s_tot[t] = run;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = s_base[d] + s_w[w][d] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        s_base[t] += s_tot[t];
#pragma unroll
        for (int j = 0; j < kSortWarps; ++j) s_w[j][t] = 0;
        __syncthreads();
    }
}

// ---- counting sort seeded by the key histogram ----------------------------
// The key histogram the cell pass counts, scanned, gives every key its
// segment [sub[k], sub[k+1]); the histogram's atomics gave every particle a
// rank among the particles of its key.  k_scatter puts (input index, key) at
// sub[k] + rank, so the order inside a segment is arbitrary; k_segsort_gather
// then sorts each segment by input index (a thread per slot), which restores
// exactly the stable order (cell, sub-cell, input index), gathers the
// positions and zeroes the key counts for the next build.  Segments longer
// than kShortSeg go to a list that k_long_segsort sorts a block per segment.
constexpr uint32_t kShortSeg = 2 * kWarp;

__global__ void k_scatter(const GridInfo* __restrict__ info, const uint32_t* __restrict__ key,
                          const uint32_t* __restrict__ rank, uint64_t n, const uint32_t* __restrict__ sub,
                          uint2* __restrict__ slots) {
    if (info->status != kGridOk) return;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = key[i];
    slots[sub[k] + rank[i]] = make_uint2((uint32_t)i, k);
}

// One thread per slot: the segment's indices are distinct, so an index's
// rank in the sorted segment is the number of the segment's indices below it;
// the thread counts them over its segment's slots (read through L1: the
// neighbouring threads walk the same lines), writes its index there and
// gathers its position.  The first slot of a segment zeroes the key's count
// and, for a long segment, lists it for k_long_segsort; the other slots of a
// long segment do nothing.
__global__ void k_segsort_gather(GridInfo* __restrict__ info, const float* __restrict__ xyz, uint32_t stride,
                                 uint64_t n, const uint32_t* __restrict__ sub, const uint2* __restrict__ slots,
                                 uint32_t* __restrict__ counts, uint32_t* __restrict__ perm,
                                 float4* __restrict__ pts, uint32_t* __restrict__ long_keys) {
    if (info->status != kGridOk) return;
    const uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint2 me = __ldg(slots + p);
    const uint32_t v = me.x, k = me.y;
    const uint32_t b = __ldg(sub + k), e = __ldg(sub + k + 1);
    if (p == b) counts[k] = 0;
    if (e - b > kShortSeg) {
        if (p == b) long_keys[atomicAdd(&info->n_long, 1u)] = k;
        return;
    }
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(slots);  // index of slot j at 2 j
    uint32_t r = 0;
#pragma unroll 4
    for (uint32_t j = b; j < e; ++j) r += __ldg(idx + 2 * (uint64_t)j) < v ? 1u : 0u;
    const float* q = xyz + (uint64_t)v * stride;
    perm[b + r] = v;
    pts[b + r] = make_float4(q[0], q[1], q[2], 0.0f);
}

// One block per long segment (grid-stride over the list): the segment's
// indices copied out of the slots, a stable LSD radix sort of them, 8 bits per
// pass, ping-ponging between the segment's ranges of tmp0 and tmp1, then the
// gather.  The indices are distinct, so the sorted segment is unique.
constexpr int kLongThreads = 256;

__global__ void __launch_bounds__(kLongThreads) k_long_segsort(const float* __restrict__ xyz, uint32_t stride,
                                                               const uint32_t* __restrict__ sub,
                                                               const uint2* __restrict__ slots,
                                                               uint32_t* __restrict__ tmp0, uint32_t* __restrict__ tmp1,
                                                               const uint32_t* __restrict__ long_keys,
                                                               const GridInfo* __restrict__ info, int passes,
                                                               uint32_t* __restrict__ perm, float4* __restrict__ pts) {
    __shared__ uint32_t s_base[256];
    __shared__ uint32_t s_w[kLongThreads / kWarp][256];
    const int t = threadIdx.x, l = t % kWarp, w = t / kWarp;
    const uint32_t lt = (1u << l) - 1u;
    const uint32_t nl = info->status == kGridOk ? info->n_long : 0u;
    for (uint32_t e = blockIdx.x; e < nl; e += gridDim.x) {
        const uint32_t k = long_keys[e];
        const uint32_t b = sub[k], m = sub[k + 1] - b;
        uint32_t* src = tmp0 + b;
        uint32_t* dst = tmp1 + b;
        for (uint32_t j = t; j < m; j += kLongThreads) src[j] = slots[b + j].x;
        __syncthreads();
        for (int p = 0; p < passes; ++p) {
            const int shift = 8 * p;
            s_base[t] = 0;
            __syncthreads();
            for (uint32_t j = t; j < m; j += kLongThreads) atomicAdd(&s_base[(src[j] >> shift) & 255u], 1u);
            __syncthreads();
            if (w == 0) {  // exclusive scan of the 256 digit counts: 8 per lane, then across the warp
                uint32_t c[8], sum = 0;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    c[j] = s_base[8 * l + j];
                    sum += c[j];
                }
                uint32_t inc = sum;
#pragma unroll
                for (int o = 1; o < kWarp; o <<= 1) {
                    const uint32_t x = __shfl_up_sync(0xffffffffu, inc, o);
                    if (l >= o) inc += x;
                }
                uint32_t run = inc - sum;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    s_base[8 * l + j] = run;
                    run += c[j];
                }
            }
            __syncthreads();
            for (uint32_t j0 = 0; j0 < m; j0 += kLongThreads) {
                const uint32_t j = j0 + t;
                const bool valid = j < m;
                const uint32_t x = valid ? src[j] : 0u;
                const uint32_t d = valid ? ((x >> shift) & 255u) : (0x10000u + l);
#pragma unroll
                for (int q = 0; q < kLongThreads / kWarp; ++q) s_w[q][t] = 0;
                __syncthreads();
                const uint32_t peers = __match_any_sync(0xffffffffu, d);
                const uint32_t rank = __popc(peers & lt);
                if (valid && rank == 0) s_w[w][d] = __popc(peers);
                __syncthreads();
                uint32_t run = 0;  // thread t: prefix over warps of digit t
#pragma unroll
                for (int q = 0; q < kLongThreads / kWarp; ++q) {
                    const uint32_t c = s_w[q][t];
                    s_w[q][t] = run;
                    run += c;
                }
                __syncthreads();
                if (valid) dst[s_base[d] + s_w[w][d] + rank] = x;
                __syncthreads();
                s_base[t] += run;
                __syncthreads();
            }
            uint32_t* sw = src;
            src = dst;
            dst = sw;
        }
        for (uint32_t j = t; j < m; j += kLongThreads) {
            const uint32_t x = src[j];
            const float* q = xyz + (uint64_t)x * stride;
            perm[b + j] = x;
            pts[b + j] = make_float4(q[0], q[1], q[2], 0.0f);
        }
        __syncthreads();
    }
}

__global__ void k_gather(const float* __restrict__ xyz, uint64_t n, uint32_t stride, const uint32_t* __restrict__ perm,
                         float4* __restrict__ out) {
    uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float* p = xyz + (uint64_t)perm[k] * stride;
    out[k] = make_float4(p[0], p[1], p[2], 0.0f);
}

// Exact-skip bound table, first level: 4x4x4 boxes per cell.
// Upper bound of the density any sample inside a bound box can reach.  Every
// cell is divided into 4x4x4 bound boxes (a quarter cell per axis); a box's
// bound is the sum over the particles of the cell's 27-neighbourhood (the
// sample's candidate set) of W at the particle's distance to the box grown by
// a slack that covers the rounding of the sample's cell assignment, inflated
// by a margin that covers the FP32 summation error of up to n terms (the
// bound's own and the sample's), and exactly 0 when no particle lies within
// the support radius of the box.  One warp per cell, lane l owns boxes l and
// l + 32: the warp loads 32 neighbourhood particles at a time (one coalesced
// 512-byte read) into its 512 bytes of shared memory, from where every lane
// reads each particle as a broadcast, and each lane adds W for its two boxes
// in registers (the order of the additions does not matter: the margin
// covers it).
//
// Once the partial sums of all 64 boxes reach `thr` (the iso density of the
// march that asked for the table), the cell stores +inf for every box and
// stops: a box whose bound is at least the iso density is never skipped, so
// +inf gives the same march at that iso and at any lower one.  The rows are
// taken centre row first, then the four sharing a face with it, then the
// diagonal ones: inside the fluid the sums reach the iso density within the
// first rows.
constexpr int kBoundWarps = 8;

__global__ void __launch_bounds__(kWarp * kBoundWarps) k_cell_bound4(GridDev g, KernelDev k, float slack, float thr,
                                                                     float* __restrict__ bound,
                                                                     float* __restrict__ fine) {
    __shared__ float4 s_pts[kBoundWarps][kWarp];
    const uint64_t ncells = (uint64_t)g.dims[0] * g.dims[1] * g.dims[2];
    const uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / kWarp;
    const int l = threadIdx.x % kWarp;
    if (c >= ncells) return;  // warp-uniform
    float4* sp = s_pts[threadIdx.x / kWarp];
    const int cc[3] = {(int)(c % (uint64_t)g.dims[0]), (int)((c / (uint64_t)g.dims[0]) % (uint64_t)g.dims[1]),
                       (int)(c / ((uint64_t)g.dims[0] * g.dims[1]))};
    // this lane's boxes b = l and l + 32 (b = ix + 4 iy + 16 iz): the same ix and
    // iy, iz and iz + 2; slab edges grown by the slack
    const int ib[4] = {l & 3, (l >> 2) & 3, l >> 4, (l >> 4) + 2};  // ix, iy, iz of box l, iz of box l + 32
    float lo[4], hi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int a = i < 3 ? i : 2;
        lo[i] = g.min[a] + ((float)cc[a] + 0.25f * (float)ib[i]) * g.cell - slack;
        hi[i] = g.min[a] + ((float)cc[a] + 0.25f * (float)(ib[i] + 1)) * g.cell + slack;
    }
    float acc0 = 0.0f, acc1 = 0.0f;
    uint32_t cnt = 0;
    bool reached = false;  // every box's sum reached thr (warp-uniform)
    const int x0 = max(cc[0] - 1, 0), x1 = min(cc[0] + 1, g.dims[0] - 1);
    // row r: 4-bit code (dy + 1) | (dz + 1) << 2 at bit 4 r; (dy, dz) = (0, 0), (-1, 0), (1, 0),
    // (0, -1), (0, 1), (-1, -1), (1, -1), (-1, 1), (1, 1)
    constexpr uint64_t kRowOrder = 0xa82091645ull;
    for (int r = 0; r < 9 && !reached; ++r) {
        const int code = (int)((kRowOrder >> (4 * r)) & 15u);
        const int y = cc[1] + (code & 3) - 1, z = cc[2] + (code >> 2) - 1;
        if (y < 0 || y >= g.dims[1] || z < 0 || z >= g.dims[2]) continue;
        const uint64_t row = ((uint64_t)z * g.dims[1] + y) * g.dims[0];
        const uint32_t b = g.sub[8 * (row + x0)], e = g.sub[8 * (row + x1) + 8];
        cnt += e - b;
        for (uint32_t j0 = b; j0 < e; j0 += kWarp) {
            const uint32_t j = j0 + (uint32_t)l;
            const float4 mine = j < e ? g.pts[j] : make_float4(0.f, 0.f, 0.f, 0.f);
            const int m = (int)min(e - j0, (uint32_t)kWarp);
            __syncwarp();
            sp[l] = mine;
            __syncwarp();
            for (int t = 0; t < m; ++t) {
                const float4 qv = sp[t];
                const float q[4] = {qv.x, qv.y, qv.z, qv.z};
                float dd[4];  // squared distance to the slab, per axis (z twice)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float d = fmaxf(fmaxf(lo[i] - q[i], q[i] - hi[i]), 0.0f);
                    dd[i] = d * d;
                }
                const float dxy = dd[0] + dd[1];
                const float d2[2] = {dxy + dd[2], dxy + dd[3]};
                if (d2[0] < k.h2) acc0 += w_in(k, d2[0]);
                if (d2[1] < k.h2) acc1 += w_in(k, d2[1]);
            }
            if (__all_sync(0xffffffffu, acc0 >= thr && acc1 >= thr)) {
                reached = true;
                break;
            }
        }
    }
    const float eps = 5.9604645e-8f;  // 2^-24
    const float n = (float)cnt;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float a = h ? acc1 : acc0;
        const float up = a * (1.0f + 16.0f * eps) * (1.0f + 4.0f * n * eps) + 32.0f * n * eps * k.sig;
        const float v = reached ? __int_as_float(0x7f800000) : ((cnt == 0 || a == 0.0f) ? 0.0f : up);
        bound[64 * c + l + 32 * h] = v;
        // the 8x8x8 table: each of the box's eight eighths starts with its bound
        const int cbx = l + 32 * h, cx = cbx & 3, cy = (cbx >> 2) & 3, cz = cbx >> 4;
        float* fb = fine + (uint64_t)kBoundBoxes * c;
#pragma unroll
        for (int f = 0; f < 8; ++f) fb[(2 * cx + (f & 1)) + 8 * (2 * cy + ((f >> 1) & 1)) + 64 * (2 * cz + (f >> 2))] = v;
    }
}

// Refinement of the bound table (8x8x8 boxes per cell, an eighth of a cell per
// axis) from its 4x4x4 first level `coarse`: k_cell_bound4 gave every eighth
// its box's bound, which stays where that is below `thr` (skipped either way),
// +inf (the cell reached thr) or 0 (no particle within reach); the eighths of
// "shell" boxes (thr <= bound < +inf: near the iso surface, where most
// evaluated samples lie) get their own sums, with the same slack and margin.
// One warp per cell: the fine boxes to sum are taken 32 at a time, one per
// lane, and each round streams the cell's 27-neighbourhood through shared
// memory as k_cell_bound4 does; a round stops once all its boxes reached thr.
// Fine box b = ix + 8 iy + 64 iz; coarse box (ix, iy, iz) / 2.
__global__ void __launch_bounds__(kWarp * kBoundWarps) k_cell_refine8(GridDev g, KernelDev k, float slack, float thr,
                                                                      const float* __restrict__ coarse,
                                                                      float* __restrict__ bound) {
    __shared__ float4 s_pts[kBoundWarps][kWarp];
    const uint64_t ncells = (uint64_t)g.dims[0] * g.dims[1] * g.dims[2];
    const uint64_t c = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) / kWarp;
    const int l = threadIdx.x % kWarp;
    // this warp's round: fine boxes 32 r .. 32 r + 31 of the cell's shell boxes
    // (rounds of one cell run in parallel warps, so a cell with many shell boxes
    // does not end the launch alone)
    const int f0 = kWarp * (int)blockIdx.y;
    if (c >= ncells) return;  // warp-uniform
    float4* sp = s_pts[threadIdx.x / kWarp];
    const float* cb = coarse + 64 * c;
    float* fb = bound + (uint64_t)kBoundBoxes * c;
    // coarse boxes l and l + 32: shell or not (the others' eighths already hold their bound)
    uint64_t shell = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const float v = cb[l + 32 * h];
        const bool sh = v >= thr && v < __int_as_float(0x7f800000);
        shell |= (uint64_t)__ballot_sync(0xffffffffu, sh) << (32 * h);
    }
    if (!shell || f0 >= 8 * __popcll(shell)) return;
    const int cc[3] = {(int)(c % (uint64_t)g.dims[0]), (int)((c / (uint64_t)g.dims[0]) % (uint64_t)g.dims[1]),
                       (int)(c / ((uint64_t)g.dims[0] * g.dims[1]))};
    const int x0 = max(cc[0] - 1, 0), x1 = min(cc[0] + 1, g.dims[0] - 1);
    constexpr uint64_t kRowOrder = 0xa82091645ull;  // centre row first, then face neighbours, then diagonals
    uint32_t cnt = 0;  // candidates of the 27-neighbourhood (for the margin)
    for (int r = 0; r < 9; ++r) {
        const int code = (int)((kRowOrder >> (4 * r)) & 15u);
        const int y = cc[1] + (code & 3) - 1, z = cc[2] + (code >> 2) - 1;
        if (y < 0 || y >= g.dims[1] || z < 0 || z >= g.dims[2]) continue;
        const uint64_t row = ((uint64_t)z * g.dims[1] + y) * g.dims[0];
        cnt += g.sub[8 * (row + x1) + 8] - g.sub[8 * (row + x0)];
    }
    const int nfine = 8 * __popcll(shell);
    {
        // this lane's fine box: the (f0 + l)-th of the shell boxes' fine boxes
        const int f = f0 + l;
        const bool live = f < nfine;
        int fbx = 0;
        if (live) {
            uint64_t m = shell;
            for (int i = 0; i < (f >> 3); ++i) m &= m - 1;  // drop the lowest (f / 8) shell boxes
            const int cbx = __ffsll((long long)m) - 1;
            const int cx = cbx & 3, cy = (cbx >> 2) & 3, cz = cbx >> 4, sub = f & 7;
            fbx = (2 * cx + (sub & 1)) + 8 * (2 * cy + ((sub >> 1) & 1)) + 64 * (2 * cz + (sub >> 2));
        }
        const int ib[3] = {fbx & 7, (fbx >> 3) & 7, fbx >> 6};
        float lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            lo[a] = g.min[a] + ((float)cc[a] + 0.125f * (float)ib[a]) * g.cell - slack;
            hi[a] = g.min[a] + ((float)cc[a] + 0.125f * (float)(ib[a] + 1)) * g.cell + slack;
        }
        float acc = 0.0f;
        bool reached = false;
        for (int r = 0; r < 9 && !reached; ++r) {
            const int code = (int)((kRowOrder >> (4 * r)) & 15u);
            const int y = cc[1] + (code & 3) - 1, z = cc[2] + (code >> 2) - 1;
            if (y < 0 || y >= g.dims[1] || z < 0 || z >= g.dims[2]) continue;
            const uint64_t row = ((uint64_t)z * g.dims[1] + y) * g.dims[0];
            const uint32_t b = g.sub[8 * (row + x0)], e = g.sub[8 * (row + x1) + 8];
            for (uint32_t j0 = b; j0 < e; j0 += kWarp) {
                const uint32_t j = j0 + (uint32_t)l;
                const float4 mine = j < e ? g.pts[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                const int m = (int)min(e - j0, (uint32_t)kWarp);
                __syncwarp();
                sp[l] = mine;
                __syncwarp();
                for (int t = 0; t < m; ++t) {
                    const float4 qv = sp[t];
                    const float q[3] = {qv.x, qv.y, qv.z};
                    float d2 = 0.0f;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float d = fmaxf(fmaxf(lo[a] - q[a], q[a] - hi[a]), 0.0f);
                        d2 += d * d;
                    }
                    if (d2 < k.h2) acc += w_in(k, d2);
                }
                if (__all_sync(0xffffffffu, !live || acc >= thr)) {
                    reached = true;
                    break;
                }
            }
        }
        if (live) {
            const float eps = 5.9604645e-8f;  // 2^-24
            const float n = (float)cnt;
            const float up = acc * (1.0f + 16.0f * eps) * (1.0f + 4.0f * n * eps) + 32.0f * n * eps * k.sig;
            fb[fbx] = reached ? __int_as_float(0x7f800000) : (acc == 0.0f ? 0.0f : up);
        }
    }
}

// Reference skip flags, Dataset.cpp:137-164, with each cell's own particle
// count as the find_neighbors_box result.
__global__ void k_ref_flags(GridDev g, float W0, uint8_t* __restrict__ flag) {
    uint64_t ncells = (uint64_t)g.dims[0] * g.dims[1] * g.dims[2];
    uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int x = (int)(c % (uint64_t)g.dims[0]);
    int y = (int)((c / (uint64_t)g.dims[0]) % (uint64_t)g.dims[1]);
    int z = (int)(c / ((uint64_t)g.dims[0] * g.dims[1]));
    float Nc = 0.0f;
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                int xx = x + dx, yy = y + dy, zz = z + dz;
                if (xx < 0 || xx >= g.dims[0] || yy < 0 || yy >= g.dims[1] || zz < 0 || zz >= g.dims[2]) continue;
                uint64_t cc = (uint64_t)xx + (uint64_t)yy * g.dims[0] + (uint64_t)zz * g.dims[0] * g.dims[1];
                const float C = 1000.0f;
                const float r = (float)(abs(dx) + abs(dy) + abs(dz));
                const float wgt = expf(-C * r);
                Nc = Nc + wgt * (float)(g.sub[8 * cc + 8] - g.sub[8 * cc]);
            }
    float rho = Nc * W0;
    flag[c] = rho > 1.0f ? 1 : 0;
}

bool ensure_buf(DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) return false;
    b.bytes = bytes;
    return true;
}

}  // namespace

GridDev grid_dev(const fm_scene* s) {
    GridDev g;
    for (int a = 0; a < 3; ++a) {
        g.min[a] = s->min[a];
        g.dims[a] = s->dims[a];
    }
    g.inv = s->inv;
    g.cell = 1.0f * s->support;
    g.pts = s->d_pts;
    g.sub = s->d_sub;
    g.nsub = (uint32_t)(8 * s->ncells + 1);
    g.bound = s->bound_valid ? s->d_bound : nullptr;
    g.flag = s->flag_valid ? s->d_flag : nullptr;
    float amax = 0.0f;
    for (int a = 0; a < 3; ++a) amax = std::max(amax, std::max(std::fabs(s->min[a]), std::fabs(s->max[a])));
    const float slack = 1.0e-4f * s->support + 1.0e-6f * amax;
    for (int a = 0; a < 3; ++a) {
        g.zlo[a] = s->min[a] - slack;
        g.zhi[a] = s->max[a] + slack;
    }
    return g;
}

uint64_t scan_words(uint64_t n) { return scan_tmp_words(n); }

void scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, uint32_t* tmp, cudaStream_t st) {
    exclusive_scan(in, out, n, tmp, st);
}

// Cell tables of a scene (sub-cell starts, bound table, reference-skip flags)
// for at least ncells cells.
static int grow_cell_tables(fm_ctx* ctx, fm_scene* s, uint64_t ncells) {
    // a bound table build of an earlier march may still be running on the side stream
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    cudaFree(s->d_sub);
    cudaFree(s->d_bound);
    cudaFree(s->d_flag);
    s->d_sub = nullptr; s->d_bound = nullptr; s->d_flag = nullptr;
    s->cell_capacity = 0;
    if (cudaMalloc(&s->d_sub, (8 * ncells + 1) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s->d_bound, ncells * kBoundBoxes * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&s->d_flag, ncells) != cudaSuccess)
        return set_err(ctx, FM_ERR_OOM, "cell table allocation failed");
    s->cell_capacity = ncells;
    return FM_OK;
}

// One build, launched for the scene's current cell capacity: the bounds pass,
// the record pass (the grid and its status into info) and, when the scene has
// cell tables, the cell keys, their scan, the counting scatter and the segment
// sorts, every one of which does nothing unless the grid fits.  No host sync.
static int launch_build(fm_ctx* ctx, fm_scene* s, const float* d_xyz, uint32_t stride, GridInfo* info) {
    cudaStream_t st = ctx->stream;
    const uint64_t n = s->n;
    const uint64_t cap = s->cell_capacity;
    uint32_t* mm = (uint32_t*)ctx->scratch[0].p;
    const bool vec3 = stride == 3 && ((uintptr_t)d_xyz & 15u) == 0;
    const uint64_t items = vec3 ? (3 * n) / 4 : n;
    uint64_t blocks = std::min<uint64_t>((items + kBoundsThreads - 1) / kBoundsThreads, (uint64_t)ctx->sm_count * 8);
    if (vec3) blocks = (std::max<uint64_t>(blocks, 1) + 2) / 3 * 3;  // grid stride a multiple of 3 float4s
    blocks = std::max<uint64_t>(blocks, 1);
    if (vec3)
        k_grid_bounds<true><<<(unsigned)blocks, kBoundsThreads, 0, st>>>(d_xyz, n, stride, mm);
    else
        k_grid_bounds<false><<<(unsigned)blocks, kBoundsThreads, 0, st>>>(d_xyz, n, stride, mm);
    k_grid_record<<<1, 1, 0, st>>>(mm, s->support, cap, info);
    FM_CUDA(ctx, cudaGetLastError());
    if (cap == 0) return FM_OK;
    const uint64_t nkeys = 8 * cap;
    uint32_t* counts = (uint32_t*)ctx->scratch[1].p;
    uint2* slots = (uint2*)ctx->scratch[2].p;
    uint32_t* rank = (uint32_t*)ctx->scratch[3].p;  // read by k_scatter, then reused as tmp0 below
    uint32_t* keys0 = (uint32_t*)ctx->scratch[7].p;
    const unsigned pblocks = (unsigned)((n + 255) / 256);
    k_cells_info<<<pblocks, 256, 0, st>>>(d_xyz, n, stride, info, s->d_cell, keys0, rank, counts);
    FM_CUDA(ctx, cudaGetLastError());
    exclusive_scan(counts, s->d_sub, nkeys + 1, (uint32_t*)ctx->scratch[6].p, st);
    FM_CUDA(ctx, cudaGetLastError());
    k_scatter<<<pblocks, 256, 0, st>>>(info, keys0, rank, n, s->d_sub, slots);
    k_segsort_gather<<<pblocks, 256, 0, st>>>(info, d_xyz, stride, n, s->d_sub, slots, counts, s->d_perm, s->d_pts,
                                              (uint32_t*)ctx->scratch[4].p);
    int ibits = 1;
    while (ibits < 32 && ((n - 1) >> ibits)) ++ibits;
    k_long_segsort<<<(unsigned)ctx->sm_count, kLongThreads, 0, st>>>(
        d_xyz, stride, s->d_sub, slots, rank, (uint32_t*)ctx->scratch[5].p, (const uint32_t*)ctx->scratch[4].p, info,
        (ibits + 7) / 8, s->d_perm, s->d_pts);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

// The grid build, one host sync at its end.  The whole chain is launched for
// the cell capacity the scene already has; the record pass computes the grid
// from the bounds on the device and the later passes read it there.  When the
// grid needs more cells than that (the first build of a scene, or a frame
// whose AABB grew) the passes after the record pass do nothing, the host grows
// the cell tables to the size the record reports and launches the chain again.
int build_grid(fm_ctx* ctx, fm_scene* s, const float* d_xyz, uint32_t stride) {
    cudaStream_t st = ctx->stream;
    const uint64_t n = s->n;
    s->bound_valid = false;
    s->flag_valid = false;
    s->occ_valid = false;
    if (!ensure_buf(ctx->scratch[2], n * sizeof(uint2)) ||     // slots: (input index, key)
        !ensure_buf(ctx->scratch[3], n * sizeof(uint32_t)) ||  // ranks, then long-segment sort temporaries
        !ensure_buf(ctx->scratch[4], n * sizeof(uint32_t)) ||  // long-segment keys
        !ensure_buf(ctx->scratch[5], n * sizeof(uint32_t)) ||  // long-segment sort temporaries
        !ensure_buf(ctx->scratch[7], n * sizeof(uint32_t)))    // keys (input order)
        return set_err(ctx, FM_ERR_OOM, "grid build scratch allocation failed");
    for (int attempt = 0; attempt < 2; ++attempt) {
        const uint64_t nkeys = 8 * s->cell_capacity;
        const size_t b0 = ctx->scratch[0].bytes, b1 = ctx->scratch[1].bytes;  // a reallocation grows them
        if (!ensure_buf(ctx->scratch[0], 128) ||                          // bounds words + grid record
            !ensure_buf(ctx->scratch[1], (nkeys + 2) * sizeof(uint32_t)) ||  // key counts
            !ensure_buf(ctx->scratch[6], scan_tmp_words(nkeys + 1) * sizeof(uint32_t)))
            return set_err(ctx, FM_ERR_OOM, "grid build scratch allocation failed");
        uint32_t* mm = (uint32_t*)ctx->scratch[0].p;
        GridInfo* info = (GridInfo*)(mm + 16);
        if (ctx->grid_scratch_dirty || ctx->scratch[0].bytes != b0 || ctx->scratch[1].bytes != b1) {
            ctx->grid_scratch_dirty = true;
            FM_CUDA(ctx, cudaMemsetAsync(mm, 0xff, 3 * sizeof(uint32_t), st));
            FM_CUDA(ctx, cudaMemsetAsync(mm + 3, 0, 4 * sizeof(uint32_t), st));
            FM_CUDA(ctx, cudaMemsetAsync(ctx->scratch[1].p, 0, ctx->scratch[1].bytes, st));
        }
        // a build that stops between its launches and the sync below leaves the
        // counts and bounds words to be set again
        ctx->grid_scratch_dirty = true;
        int rc = launch_build(ctx, s, d_xyz, stride, info);
        if (rc != FM_OK) return rc;
        GridInfo* h = (GridInfo*)ctx->h_pinned_small;
        FM_CUDA(ctx, cudaMemcpyAsync(h, info, sizeof(GridInfo), cudaMemcpyDeviceToHost, st));
        FM_CUDA(ctx, cudaStreamSynchronize(st));
        // every pass has run: the segment sort zeroed the counts (or the cell
        // pass did not touch them) and the bounds words are back to their start
        ctx->grid_scratch_dirty = false;
        const GridInfo gi = *h;
        if (gi.status == kGridNonFinite)
            return set_err(ctx, FM_ERR_INVALID, "particle positions contain non-finite values");
        if (gi.status == kGridExtent)
            return set_err(ctx, FM_ERR_INVALID, "grid extent / support radius out of range");
        if (gi.status == kGridTooMany)
            return set_err(ctx, FM_ERR_INVALID, "grid would exceed 2^28 cells: support radius too small for the extent");
        if (gi.status == kGridOverCapacity) {
            if ((rc = grow_cell_tables(ctx, s, gi.ncells)) != FM_OK) return rc;
            continue;
        }
        if (gi.status != kGridOk) return set_err(ctx, FM_ERR_CUDA, "grid build returned an unknown status");
        for (int a = 0; a < 3; ++a) {
            s->min[a] = gi.g.min[a];
            s->max[a] = gi.max[a];
            s->dims[a] = gi.g.dims[a];
        }
        s->inv = gi.g.inv;
        s->ncells = gi.ncells;
        return FM_OK;
    }
    return set_err(ctx, FM_ERR_CUDA, "grid build: cell capacity still short after growing the tables");
}

// The bound table stores +inf for the boxes of a cell once all their sums
// reached the march's iso density, so it serves marches at that iso or a
// lower one; a march at a higher iso builds it again (in place: a march still
// reading it sees one valid bound or the other in every box).
static float bound_thr(float iso) { return (iso > 0.0f && std::isfinite(iso)) ? iso : INFINITY; }

bool bound_stale(const fm_scene* s, float iso) { return !(s->bound_valid && bound_thr(iso) <= s->bound_iso); }

static float bound_slack(const fm_scene* s) {
    float amax = 0.0f;
    for (int a = 0; a < 3; ++a) amax = std::max(amax, std::max(std::fabs(s->min[a]), std::fabs(s->max[a])));
    return 1.0e-4f * s->support + 1.0e-6f * amax;
}

int ensure_bound(fm_ctx* ctx, fm_scene* s, cudaStream_t st, float iso) {
    const float thr = bound_thr(iso);
    if (!bound_stale(s, iso)) return FM_OK;
    if (!ensure_buf(s->coarse, s->ncells * 64 * sizeof(float)))
        return set_err(ctx, FM_ERR_OOM, "bound table allocation failed");
    GridDev g = grid_dev(s);
    KernelDev k = make_kernel(s->support);
    const uint64_t blocks = (s->ncells + kBoundWarps - 1) / kBoundWarps;
    k_cell_bound4<<<(unsigned)blocks, kWarp * kBoundWarps, 0, st>>>(g, k, bound_slack(s), thr, (float*)s->coarse.p,
                                                                    s->d_bound);
    FM_CUDA(ctx, cudaGetLastError());
    s->bound_valid = true;
    s->bound_iso = thr;
    s->bound_fine = false;
    // the second level right behind the first, on the same stream: at 1080p it
    // costs 0.74 ms and saves about 1.4 ms of the march that reads it
    return refine_bound(ctx, s, st);
}

// Second level: the shell boxes of the first (iso <= bound < inf) split into
// eighths, a warp per (cell, round of 32 eighths).
int refine_bound(fm_ctx* ctx, fm_scene* s, cudaStream_t st) {
    if (!s->bound_valid || s->bound_fine) return FM_OK;
    GridDev g = grid_dev(s);
    KernelDev k = make_kernel(s->support);
    const uint64_t blocks = (s->ncells + kBoundWarps - 1) / kBoundWarps;
    // y: the round (64 shell boxes x 8 fine boxes / 32 lanes = 16 at most)
    const dim3 grid((unsigned)blocks, 64 * 8 / kWarp);
    k_cell_refine8<<<grid, kWarp * kBoundWarps, 0, st>>>(g, k, bound_slack(s), s->bound_iso,
                                                         (const float*)s->coarse.p, s->d_bound);
    FM_CUDA(ctx, cudaGetLastError());
    s->bound_fine = true;
    return FM_OK;
}

int ensure_flags(fm_ctx* ctx, fm_scene* s, cudaStream_t st) {
    if (s->flag_valid) return FM_OK;
    GridDev g = grid_dev(s);
    KernelDev k = make_kernel(s->support);
    k_ref_flags<<<(unsigned)((s->ncells + 255) / 256), 256, 0, st>>>(g, k.sig, s->d_flag);
    FM_CUDA(ctx, cudaGetLastError());
    s->flag_valid = true;
    return FM_OK;
}

}  // namespace fm

// ============================================================================
// Grid build that allocates nothing: fm_grid_build_noalloc
// ============================================================================
//
// For callers that must not allocate device memory: code that runs where
// cudaMalloc is not allowed or not wanted (a renderer that reserves all of its
// memory up front, a plugin living inside a host application's memory
// budget).  Same kernels and same results as the grid build of
// fm_scene_create; the caller passes every output buffer, and the scratch the
// build needs lives in one file-scope device array:
//   * the AABB words, the radix-sort histograms and the scan temporaries in
//     g_noalloc_scratch (kNoAllocWords words, about 1.1 MB, which every device
//     that loads this library keeps until the process exits);
//   * the sort keys and values in the caller's sorted_xyzw buffer (4n words),
//     which holds them until the final gather writes the sorted positions.
// Limits: n <= 2^21 particles and n_cells <= 2^21.  Every call shares the
// scratch array, so calls that overlap on the GPU (other streams, other host
// threads) race; serialise them.  The array keeps the last call's contents;
// the AABB words are cleared at the start of each call and everything else is
// fully rewritten before it is read.
//
// The array's device address differs per CUDA context (the library's module
// is loaded into each context that uses it), and a host application may run
// this call under a driver-API context of its own rather than the device's
// primary context.  So the address is looked up once per context, with that
// context current, and cached under the context's unique id (cuCtxGetId,
// reached through the runtime's driver entry points, so the library does not
// link libcuda itself).

#include <cuda.h>

#include <mutex>
#include <unordered_map>

namespace fm {
namespace {

constexpr uint64_t kNoAllocMaxParticles = 1ull << 21;
constexpr uint64_t kNoAllocMaxCells = 1ull << 21;
constexpr uint64_t kNoAllocAabbWords = 64;
constexpr uint64_t kNoAllocHistWords = 256 * ((kNoAllocMaxParticles + kSortTile - 1) / kSortTile);
constexpr uint64_t kNoAllocScanWords = 16384;  // >= scan_tmp_words(8 * kNoAllocMaxCells + 1)
constexpr uint64_t kNoAllocWords = kNoAllocAabbWords + kNoAllocHistWords + kNoAllocScanWords;

__device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

std::mutex g_noalloc_mu;
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;
constexpr size_t kNoAllocCacheMax = 4096;  // contexts remembered; beyond it the address is looked up per call
std::unordered_map<unsigned long long, uint32_t*> g_noalloc_addr;

// Unique id of the calling thread's current CUDA context (0 when none is current).
int current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return FM_ERR_CUDA;
        g_ctx_get_current = (PfnCtxGetCurrent)f1;
        g_ctx_get_id = (PfnCtxGetId)f2;
    }
    CUcontext c = nullptr;
    if (g_ctx_get_current(&c) != CUDA_SUCCESS) return FM_ERR_CUDA;
    *id = 0;
    if (c && g_ctx_get_id(c, id) != CUDA_SUCCESS) return FM_ERR_CUDA;
    return FM_OK;
}

// Device address of g_noalloc_scratch in the current context (a host-side
// reference to the symbol is not a device address).
int noalloc_scratch(uint32_t** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    unsigned long long id = 0;
    if (current_context_id(&id) != FM_OK) return FM_ERR_CUDA;
    if (id != 0) {
        auto it = g_noalloc_addr.find(id);
        if (it != g_noalloc_addr.end()) {
            *out = it->second;
            return FM_OK;
        }
    }
    // with no context current yet, this lookup makes the device's primary context current
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return FM_ERR_CUDA;
    if (id == 0 && current_context_id(&id) != FM_OK) return FM_ERR_CUDA;
    if (id != 0 && g_noalloc_addr.size() < kNoAllocCacheMax) g_noalloc_addr[id] = (uint32_t*)p;
    *out = (uint32_t*)p;
    return FM_OK;
}

// True for memory of `dev` itself or managed memory: the kernels of this call
// read and write through these pointers.
bool on_device(const void* ptr, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeManaged || (a.type == cudaMemoryTypeDevice && a.device == dev);
}

}  // namespace
}  // namespace fm

extern "C" int fm_grid_build_noalloc(const float* xyz, uint64_t n, uint32_t stride, float support_radius,
                                     float* sorted_xyzw, uint32_t* cell, uint32_t* sorted_index, uint32_t* sub_start,
                                     uint64_t sub_start_capacity, fm_grid_info* info, void* stream) {
    using namespace fm;
    if (!xyz || !sorted_xyzw || !cell || !sorted_index || !sub_start || !info) return FM_ERR_INVALID;
    if (n == 0 || n > kNoAllocMaxParticles || stride < 3) return FM_ERR_INVALID;
    if (!(support_radius > 0.0f) || !std::isfinite(support_radius)) return FM_ERR_INVALID;
    if (((uintptr_t)sorted_xyzw & 15u) != 0) return FM_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FM_ERR_CUDA;
    uint32_t* scratch = nullptr;
    if (noalloc_scratch(&scratch) != FM_OK) return FM_ERR_CUDA;
    for (const void* p : {(const void*)xyz, (const void*)sorted_xyzw, (const void*)cell, (const void*)sorted_index,
                          (const void*)sub_start})
        if (!on_device(p, dev)) return FM_ERR_INVALID;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    uint32_t* mm = scratch;
    uint32_t* hist = scratch + kNoAllocAabbWords;
    uint32_t* tmp = hist + kNoAllocHistWords;
#define FM_NA(call)                                  \
    do {                                             \
        if ((call) != cudaSuccess) return FM_ERR_CUDA; \
    } while (0)
    // 1. AABB (exact min/max) -> host
    FM_NA(cudaMemsetAsync(mm, 0xff, 3 * sizeof(uint32_t), st));
    FM_NA(cudaMemsetAsync(mm + 3, 0, 4 * sizeof(uint32_t), st));
    {
        unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 8);
        k_aabb<<<std::max(1u, blocks), 256, 0, st>>>(xyz, n, stride, mm);
        FM_NA(cudaGetLastError());
    }
    uint32_t h[7];
    FM_NA(cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, st));
    FM_NA(cudaStreamSynchronize(st));
    if (h[6] != 0) return FM_ERR_INVALID;  // non-finite positions
    // 2. grid parameters, in the reference's FP32 order (Dataset.cpp:89-104)
    const float pad = 1.0f * support_radius;
    const float cellw = 1.0f * support_radius;
    GridParams gp;
    uint64_t ncells = 1;
    for (int a = 0; a < 3; ++a) {
        const float mn = ord2f(h[a]), mx = ord2f(h[3 + a]);
        info->max[a] = mx + pad;
        info->min[a] = mn - pad;
        const float d = std::ceil((info->max[a] - info->min[a]) / cellw);
        if (!(d >= 1.0f && d < 1.0e6f)) return FM_ERR_INVALID;
        info->dims[a] = (int)d;
        gp.min[a] = info->min[a];
        gp.dims[a] = info->dims[a];
        ncells *= (uint64_t)info->dims[a];
    }
    gp.inv = 1.0f / cellw;
    info->cell_width = cellw;
    info->inv_cell_width = gp.inv;
    info->pad = 0;
    info->n_particles = n;
    info->n_cells = ncells;
    const uint64_t nkeys = 8 * ncells;
    if (ncells > kNoAllocMaxCells || sub_start_capacity < nkeys + 1) return FM_ERR_INVALID;
    // 3. cells, keys, key histogram (the histogram is counted in sub_start)
    uint32_t* keys0 = (uint32_t*)sorted_xyzw;
    uint32_t* kbuf[2] = {keys0 + n, keys0 + 2 * n};
    uint32_t* vbuf[2] = {sorted_index, keys0 + 3 * n};
    FM_NA(cudaMemsetAsync(sub_start, 0, (nkeys + 1) * sizeof(uint32_t), st));
    k_cells<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(xyz, n, stride, gp, cell, keys0, sub_start);
    FM_NA(cudaGetLastError());
    exclusive_scan(sub_start, sub_start, nkeys + 1, tmp, st);
    // 4. stable LSD radix sort of (key, input index), the last pass landing in sorted_index
    const uint64_t nblk = (n + kSortTile - 1) / kSortTile;
    const uint64_t hist_n = 256 * nblk;
    int bits = 1;
    while (bits < 32 && ((nkeys - 1) >> bits)) ++bits;
    const int passes = (bits + 7) / 8;
    int cur = (passes % 2 == 1) ? 0 : 1;
    const uint32_t* kin = keys0;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < passes; ++p) {
        const int shift = 8 * p;
        k_radix_hist<<<(unsigned)nblk, kSortThreads, 0, st>>>(kin, n, shift, (uint32_t)nblk, hist);
        exclusive_scan(hist, hist, hist_n, tmp, st);
        k_radix_scatter<<<(unsigned)nblk, kSortThreads, 0, st>>>(kin, vin, kbuf[cur], vbuf[cur], n, shift,
                                                               (uint32_t)nblk, hist);
        FM_NA(cudaGetLastError());
        kin = kbuf[cur];
        vin = vbuf[cur];
        cur ^= 1;
    }
    // 5. gather the sorted positions (overwrites the key/value temporaries)
    k_gather<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(xyz, n, stride, sorted_index, (float4*)sorted_xyzw);
    FM_NA(cudaGetLastError());
#undef FM_NA
    return FM_OK;
}
