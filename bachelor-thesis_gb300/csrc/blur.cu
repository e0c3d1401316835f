// blur.cu -- the reference's depth Gaussian blur pass.
//
// GaussRenderPass (src/app/AdvancedRenderer/GaussRenderPass.cpp:13-57, 347-355)
// with gauss.frag: a (2N+1)^2 kernel of weights exp(-r^2 / 2) at the integer
// offsets (i, j), r = |(i, j)|, normalised to sum 1 (ComputeGaussKernel), and
// per output pixel the sum over i = -N..N (outer) and j = -N..N (inner) of
// weight(|i|, |j|) times the depth texture sampled at the pixel's UV plus
// (i, j) * (Spread / W, Spread / H).  The texture is the splat depth buffer
// with the sampler of BilateralBuffer.cpp:244-258: linear filtering,
// clamp-to-edge.
//
// Restated here in FP32 with every multiply and add rounded separately:
// UV = ((x + 0.5) / W, (y + 0.5) / H); linear filtering as the Vulkan
// specification defines it (texel coordinate u W - 1/2, its floor and
// fraction, the fraction kept to 8 sub-texel bits as GPUs report them, the
// four texels clamped to the edge); the kernel weights computed on the host
// in ComputeGaussKernel's order.  With Spread = 1 every tap lands on a texel
// centre and reads that texel exactly.  One thread per output pixel; the taps
// are L1 / L2 reads of the (small, L2-resident) depth buffer.

#include <cmath>

#include "fm_internal.cuh"

namespace fm {

constexpr int kBlurMaxN = 31;  // gauss.frag MAX_KERNEL_N 32; the UI slider stops at 31

// ComputeGaussKernel (GaussRenderPass.cpp:24-57): out[j + i (N + 1)] for
// i, j = 0..N, divided by the sum over the whole (2N+1)^2 grid.
void gauss_weights(int N, float* out) {
    const float e = 2.71828182845904523536f;
    float sum = 0.0f;
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j <= N; ++j) {
            const float r = std::sqrt((float)i * (float)i + (float)j * (float)j);
            const float y = std::pow(e, -0.5f * r * r);
            out[j + i * (N + 1)] = y;
            if (i == 0 && j == 0)
                sum += y;
            else if (i != 0 && j != 0)
                sum += 4.0f * y;
            else
                sum += 2.0f * y;
        }
    for (int k = 0; k < (N + 1) * (N + 1); ++k) out[k] /= sum;
}

namespace {

// Launch arguments, the weights included (4 KB at most: each launch carries
// its own, so concurrent blurs with different N do not share state).
struct BlurArgs {
    const float* in;
    float* out;
    int W, Hh, N;
    float tw, th;  // Spread / W, Spread / H (GaussRenderPass::UpdateUniforms)
    float w[(kBlurMaxN + 1) * (kBlurMaxN + 1)];
};

// Linear filtering of the depth texture at (s, t), clamp-to-edge.
__device__ __forceinline__ float sample_linear(const BlurArgs& a, float s, float t) {
    const float u = s * (float)a.W - 0.5f, v = t * (float)a.Hh - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    float al = u - fu, be = v - fv;
    al = rintf(al * 256.0f) * 0.00390625f;  // 8 sub-texel bits
    be = rintf(be * 256.0f) * 0.00390625f;
    const int i0 = (int)fmaxf(fminf(fu, (float)a.W), -1.0f), j0 = (int)fmaxf(fminf(fv, (float)a.Hh), -1.0f);
    const int x0 = min(max(i0, 0), a.W - 1), x1 = min(max(i0 + 1, 0), a.W - 1);
    const int y0 = min(max(j0, 0), a.Hh - 1), y1 = min(max(j0 + 1, 0), a.Hh - 1);
    const float t00 = __ldg(a.in + (size_t)y0 * a.W + x0), t10 = __ldg(a.in + (size_t)y0 * a.W + x1);
    const float t01 = __ldg(a.in + (size_t)y1 * a.W + x0), t11 = __ldg(a.in + (size_t)y1 * a.W + x1);
    const float ia = 1.0f - al, ib = 1.0f - be;
    return (ia * ib) * t00 + (al * ib) * t10 + (ia * be) * t01 + (al * be) * t11;
}

__global__ void k_depth_blur(const __grid_constant__ BlurArgs a) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= a.W || y >= a.Hh) return;
    const float u0 = ((float)x + 0.5f) / (float)a.W, v0 = ((float)y + 0.5f) / (float)a.Hh;
    float sum = 0.0f;
    for (int i = -a.N; i <= a.N; ++i) {
        const float s = u0 + (float)i * a.tw;
        const int wi = (i < 0 ? -i : i) * (a.N + 1);
        for (int j = -a.N; j <= a.N; ++j) {
            const float t = v0 + (float)j * a.th;
            sum = sum + a.w[wi + (j < 0 ? -j : j)] * sample_linear(a, s, t);
        }
    }
    a.out[(size_t)y * a.W + x] = sum;
}

}  // namespace
}  // namespace fm

using namespace fm;

extern "C" int fm_depth_blur(fm_ctx* ctx, const float* depth, float* out, int32_t width, int32_t height, int32_t n,
                             float spread, int mem, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!depth || !out) return set_err(ctx, FM_ERR_INVALID, "NULL buffer");
    if (width <= 0 || height <= 0 || (int64_t)width * height > (1ll << 31))
        return set_err(ctx, FM_ERR_INVALID, "image size out of range");
    if (n < 0 || n > kBlurMaxN) return set_err(ctx, FM_ERR_INVALID, "kernel half-width must be in [0, 31]");
    if (!(spread > 0.0f) || !std::isfinite(spread)) return set_err(ctx, FM_ERR_INVALID, "spread must be positive");
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const size_t bytes = (size_t)width * height * sizeof(float);
    const float* din = depth;
    float* dout = out;
    if (mem == FM_MEM_HOST) {
        if (!grow_buf(ctx->blur_in, bytes) || !grow_buf(ctx->blur_out, bytes))
            return set_err(ctx, FM_ERR_OOM, "blur buffer allocation failed");
        FM_CUDA(ctx, cudaMemcpyAsync(ctx->blur_in.p, depth, bytes, cudaMemcpyHostToDevice, st));
        din = (const float*)ctx->blur_in.p;
        dout = (float*)ctx->blur_out.p;
    }
    BlurArgs a;
    a.in = din;
    a.out = dout;
    a.W = width;
    a.Hh = height;
    a.N = n;
    a.tw = spread / (float)width;
    a.th = spread / (float)height;
    gauss_weights(n, a.w);
    const dim3 block(32, 8), grid((unsigned)((width + 31) / 32), (unsigned)((height + 7) / 8));
    k_depth_blur<<<grid, block, 0, st>>>(a);
    FM_CUDA(ctx, cudaGetLastError());
    if (mem == FM_MEM_HOST) {
        FM_CUDA(ctx, cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, st));
        FM_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return FM_OK;
}
