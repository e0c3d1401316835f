// splat.cu -- particle sphere-splat depth (the reference's depth pass).
//
// The reference rasterises one camera-facing quad of half size R per particle
// (AdvancedRenderer.cpp:447-485) with depth.vert/depth.frag:
//   UV in [-1,1]^2, discard l2 = |UV|^2 > 1,
//   depth = proj(view_pos - R * (0, 0, cos(pi/2 * sqrt(l2)))).z / w,
// into a D32 buffer cleared to 1.0 with a LESS test (DepthRenderPass.cpp:54,179).
// The quad lies in the view-space plane z = view_z(p), so for a pixel centre
// the quad point is (ndc * z / P00, ndc * z / P11) and UV follows directly.
// This kernel evaluates exactly that per covered pixel centre, in the same
// FP32 operation order as the CPU oracle, and keeps the minimum with an
// atomicMin on the float bits (depths are in [0, 1), where the uint order is
// the float order).  cos is a degree-16 Taylor polynomial (coefficients
// 1/(2k)! as exact float literals), identical in the oracle.
//
// Memory: reads 16 B per particle (cell-sorted float4), one 4 B atomic per
// covered pixel.  Particles whose disc is not fully in front of the camera
// (view z - R <= 0) and fragments outside [0, 1) are dropped.

#include <cuda_runtime.h>

#include "fm_internal.cuh"

namespace fm {
namespace {

struct SplatArgs {
    float V[16];
    float P00, P11, P22, P32, P23, P33;
    float R, invR;
    float twoWinv, twoHinv;
    int W, Hh;
};

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

__global__ void __launch_bounds__(256) k_splat(const float4* __restrict__ pts, uint64_t n, SplatArgs a,
                                               uint32_t* __restrict__ depth) {
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 q = pts[i];
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float add0 = a.V[0 * 4 + r] * q.x + a.V[1 * 4 + r] * q.y;
        float add1 = a.V[2 * 4 + r] * q.z + a.V[3 * 4 + r] * 1.0f;
        c[r] = add0 + add1;
    }
    const float cx = c[0] / c[3], cy = c[1] / c[3], cz = c[2] / c[3];
    const float R = a.R;
    if (!(cz - R > 0.0f)) return;
    float nx0 = a.P00 * (cx - R) / cz, nx1 = a.P00 * (cx + R) / cz;
    float ny0 = a.P11 * (cy - R) / cz, ny1 = a.P11 * (cy + R) / cz;
    float xa = fminf(nx0, nx1), xb = fmaxf(nx0, nx1);
    float ya = fminf(ny0, ny1), yb = fmaxf(ny0, ny1);
    float fx0 = floorf((xa + 1.0f) * 0.5f * (float)a.W - 0.5f) - 1.0f;
    float fx1 = ceilf((xb + 1.0f) * 0.5f * (float)a.W - 0.5f) + 1.0f;
    float fy0 = floorf((ya + 1.0f) * 0.5f * (float)a.Hh - 0.5f) - 1.0f;
    float fy1 = ceilf((yb + 1.0f) * 0.5f * (float)a.Hh - 0.5f) + 1.0f;
    if (fx1 < 0.0f || fy1 < 0.0f || fx0 > (float)(a.W - 1) || fy0 > (float)(a.Hh - 1)) return;
    int x0 = max(0, (int)fmaxf(fx0, -1.0f)), x1 = min(a.W - 1, (int)fminf(fx1, (float)a.W));
    int y0 = max(0, (int)fmaxf(fy0, -1.0f)), y1 = min(a.Hh - 1, (int)fminf(fy1, (float)a.Hh));
    for (int y = y0; y <= y1; ++y) {
        float ny = ((float)y + 0.5f) * a.twoHinv - 1.0f;
        float vy = (ny * cz) / a.P11;
        float vv = (vy - cy) * a.invR;
        for (int x = x0; x <= x1; ++x) {
            float nx = ((float)x + 0.5f) * a.twoWinv - 1.0f;
            float vx = (nx * cz) / a.P00;
            float uu = (vx - cx) * a.invR;
            float l2 = uu * uu + vv * vv;
            if (l2 > 1.0f) continue;
            float off = cos_poly(1.57079632679f * sqrtf(l2));
            float zv = cz - R * off;
            float d = (a.P22 * zv + a.P32) / (a.P23 * zv + a.P33);
            if (!(d >= 0.0f && d < 1.0f)) continue;
            d = d + 0.0f;
            uint32_t* dst = depth + (uint64_t)y * a.W + x;
            uint32_t bits = __float_as_uint(d);
            if (bits < *((volatile uint32_t*)dst)) atomicMin(dst, bits);
        }
    }
}

}  // namespace

int launch_splat(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, float* d_depth, cudaStream_t st) {
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
    uint64_t npx = (uint64_t)cam->width * cam->height;
    k_fill<<<(unsigned)((npx + 255) / 256), 256, 0, st>>>((uint32_t*)d_depth, npx, 0x3f800000u);
    if (s->n > 0) k_splat<<<(unsigned)((s->n + 255) / 256), 256, 0, st>>>(s->d_pts, s->n, a, (uint32_t*)d_depth);
    FM_CUDA(ctx, cudaGetLastError());
    return FM_OK;
}

}  // namespace fm
