// api.cu -- the C ABI of libfluidmarch (include/fluidmarch.h).
//
// Host side of the drop-in for the reference's RayMarcher / Frame classes
// (src/app/AdvancedRenderer/RayMarcher.{h,cpp}, src/app/Dataset.{h,cpp}).
// Contexts own a non-blocking CUDA stream, a device status word that kernels
// set on internal errors, counters, and staging buffers for host pointers.
// Every entry point validates its arguments first and returns an FM_* status;
// nothing here computes on the CPU.

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>

#include "fm_internal.cuh"

namespace fm {

int set_err(fm_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_err(fm_ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_err(ctx, FM_ERR_OOM, m);
    return set_err(ctx, FM_ERR_CUDA, m);
}

namespace {

bool grow(DevBuf& b, size_t bytes) {
    if (b.bytes >= bytes) return true;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) return false;
    b.bytes = bytes;
    return true;
}

cudaStream_t pick(fm_ctx* ctx, void* stream) { return stream ? (cudaStream_t)stream : ctx->stream; }

}  // namespace

static bool finite16(const float* m) {
    for (int i = 0; i < 16; ++i)
        if (!std::isfinite(m[i])) return false;
    return true;
}

int check_camera(fm_ctx* ctx, const fm_camera* c, bool need_splat) {
    if (!c) return set_err(ctx, FM_ERR_INVALID, "camera is NULL");
    if (c->width <= 0 || c->height <= 0) return set_err(ctx, FM_ERR_INVALID, "image size must be positive");
    if ((uint64_t)c->width * (uint64_t)c->height > (1ull << 31))
        return set_err(ctx, FM_ERR_INVALID, "image larger than 2^31 pixels");
    if (c->height > 65535 * 8) return set_err(ctx, FM_ERR_INVALID, "image height too large");
    if (!finite16(c->inv_proj_view) || !std::isfinite(c->position[0]) || !std::isfinite(c->position[1]) ||
        !std::isfinite(c->position[2]))
        return set_err(ctx, FM_ERR_INVALID, "camera matrix or position is not finite");
    if (need_splat) {
        if (!finite16(c->view) || !finite16(c->proj))
            return set_err(ctx, FM_ERR_INVALID, "view or projection matrix is not finite");
        const float* P = c->proj;
        // perspective without skew or offset: only P00, P11, P22, P23, P32, P33 may be non-zero
        const int zero[] = {1, 2, 3, 4, 6, 7, 8, 9, 12, 13};
        for (int i : zero)
            if (P[i] != 0.0f)
                return set_err(ctx, FM_ERR_INVALID, "projection must be a perspective matrix without skew or offset");
        if (P[0] == 0.0f || P[5] == 0.0f) return set_err(ctx, FM_ERR_INVALID, "degenerate projection matrix");
        const float* V = c->view;
        if (V[3] != 0.0f || V[7] != 0.0f || V[11] != 0.0f || V[15] != 1.0f)
            return set_err(ctx, FM_ERR_INVALID, "view matrix must be affine (last row 0 0 0 1)");
    }
    return FM_OK;
}

int check_params(fm_ctx* ctx, const fm_march_params* p) {
    if (!p) return set_err(ctx, FM_ERR_INVALID, "march params are NULL");
    if (!std::isfinite(p->iso_density)) return set_err(ctx, FM_ERR_INVALID, "iso density is not finite");
    if (!(p->step_size > 0.0f) || !std::isfinite(p->step_size))
        return set_err(ctx, FM_ERR_INVALID, "step size must be positive and finite");
    if (p->max_steps < 0) return set_err(ctx, FM_ERR_INVALID, "max_steps must be >= 0");
    if (p->bisect_iters < 0 || p->bisect_iters > 64) return set_err(ctx, FM_ERR_INVALID, "bisect_iters must be in [0, 64]");
    if (p->skip_mode < FM_SKIP_OFF || p->skip_mode > FM_SKIP_REFERENCE)
        return set_err(ctx, FM_ERR_INVALID, "unknown skip mode");
    if (p->flags & ~(FM_MARCH_EXTERNAL_DEPTH | FM_MARCH_PROPOSAL | FM_MARCH_ANISOTROPIC))
        return set_err(ctx, FM_ERR_INVALID, "unknown march flags");
    if (p->flags & FM_MARCH_ANISOTROPIC) {
        if (p->flags & FM_MARCH_PROPOSAL)
            return set_err(ctx, FM_ERR_INVALID, "the anisotropic march takes no proposal");
    }
    return FM_OK;
}

}  // namespace fm

using namespace fm;

extern "C" {

int fm_version(void) { return 10000; }

int fm_create(fm_ctx** out, int device) {
    if (!out) return FM_ERR_INVALID;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return FM_ERR_CUDA;
    if (device < 0 || device >= count) return FM_ERR_INVALID;
    fm_ctx* ctx = new (std::nothrow) fm_ctx();
    if (!ctx) return FM_ERR_OOM;
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        if (ctx->stream) cudaStreamDestroy(ctx->stream);
        delete ctx;
        return FM_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_jfork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_jjoin, cudaEventDisableTiming) != cudaSuccess) {
        fm_destroy(ctx);
        return FM_ERR_CUDA;
    }
    if (cudaMalloc(&ctx->d_status, 64) != cudaSuccess || cudaMalloc(&ctx->d_stats, fm::kStatSlots * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&ctx->d_work, fm::kWorkSlots * 32 * sizeof(unsigned int)) != cudaSuccess ||
        cudaHostAlloc(&ctx->h_pinned_small, 256, cudaHostAllocDefault) != cudaSuccess) {
        fm_destroy(ctx);
        return FM_ERR_OOM;
    }
    cudaMemset(ctx->d_status, 0, 64);
    cudaMemset(ctx->d_stats, 0, fm::kStatSlots * sizeof(unsigned long long));
    cudaDeviceSynchronize();
    *out = ctx;
    return FM_OK;
}

static void scene_free(fm_scene* s) {
    cudaFree(s->d_pts);
    cudaFree(s->d_cell);
    cudaFree(s->d_perm);
    cudaFree(s->d_sub);
    cudaFree(s->d_bound);
    cudaFree(s->coarse.p);
    cudaFree(s->d_flag);
    cudaFree(s->d_occ);
    delete s;
}

void fm_destroy(fm_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    // batches and scenes still alive die with their context (their handles become invalid)
    destroy_batches(ctx);
    for (fm_scene* s : ctx->scenes) scene_free(s);
    ctx->scenes.clear();
    for (auto& b : ctx->stage) cudaFree(b.p);
    for (auto& b : ctx->scratch) cudaFree(b.p);
    cudaFree(ctx->d_status);
    cudaFree(ctx->d_stats);
    cudaFree(ctx->d_work);
    cudaFree(ctx->longq.p);
    cudaFree(ctx->aniso_list.p);
    cudaFree(ctx->longq2.p);
    cudaFree(ctx->rg_keys.p);
    cudaFree(ctx->rg_tmp.p);
    cudaFree(ctx->rg_order.p);
    cudaFree(ctx->hiz.p);
    cudaFree(ctx->splat_list.p);
    cudaFree(ctx->prop_ivl.p);
    cudaFree(ctx->file_rec.p);
    cudaFree(ctx->blur_in.p);
    cudaFree(ctx->blur_out.p);
    cudaFree(ctx->file_xyz.p);
    cudaFree(ctx->prop_scratch.p);
    cudaFree(ctx->prop_low.p);
    cudaFree(ctx->prop_judge.p);
    cudaFree(ctx->judge_z.p);
    cudaFree(ctx->judge_ref.p);
    cudaFree(ctx->judge_test.p);
    cudaFree(ctx->judge_acc.p);
    cudaFree(ctx->judge_longq.p);
    if (ctx->h_pinned_small) cudaFreeHost(ctx->h_pinned_small);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->ev_jfork) cudaEventDestroy(ctx->ev_jfork);
    if (ctx->ev_jjoin) cudaEventDestroy(ctx->ev_jjoin);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* fm_last_error(const fm_ctx* ctx) {
    if (!ctx) return "no context";
    return ctx->err.c_str();
}

const char* fm_last_error_string(const fm_ctx* ctx) { return fm_last_error(ctx); }

void* fm_stream(fm_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int fm_sync(fm_ctx* ctx, int timeout_ms) {
    if (!ctx) return FM_ERR_INVALID;
    cudaSetDevice(ctx->device);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return cuda_err(ctx, e, "cudaStreamQuery");
        if (timeout_ms >= 0 &&
            std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return set_err(ctx, FM_ERR_TIMEOUT, "fm_sync: timed out waiting for the stream");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    unsigned int* h = (unsigned int*)ctx->h_pinned_small;
    FM_CUDA(ctx, cudaMemcpy(h, ctx->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost));
    if (h[0] != 0) {
        unsigned int code = h[0];
        cudaMemset(ctx->d_status, 0, sizeof(unsigned int));
        return set_err(ctx, FM_ERR_DEVICE, "kernel status word set: " + std::to_string(code) +
                                               " (bit 1: reference skip loop reached its iteration cap;"
                                               " bit 2: a march index guard fired)");
    }
    return FM_OK;
}

int fm_query(fm_ctx* ctx) {
    if (!ctx) return -FM_ERR_INVALID;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaStreamQuery(ctx->stream);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    cuda_err(ctx, e, "cudaStreamQuery");
    return -FM_ERR_CUDA;
}

int fm_host_alloc(fm_ctx* ctx, size_t bytes, void** out) {
    if (!ctx || !out) return FM_ERR_INVALID;
    cudaSetDevice(ctx->device);
    if (cudaHostAlloc(out, bytes, cudaHostAllocMapped) != cudaSuccess) {
        *out = nullptr;
        return set_err(ctx, FM_ERR_OOM, "cudaHostAlloc failed");
    }
    void* d = nullptr;
    if (cudaHostGetDevicePointer(&d, *out, 0) != cudaSuccess) {
        cudaGetLastError();
        d = nullptr;  // not mapped: outputs placed here are staged as usual
    }
    if (d && bytes) ctx->host_allocs[(uintptr_t)*out] = {bytes, d};
    return FM_OK;
}

void fm_host_free(fm_ctx* ctx, void* p) {
    if (ctx) {
        cudaSetDevice(ctx->device);
        // a kernel on any stream may still be writing into the block
        cudaDeviceSynchronize();
        ctx->host_allocs.erase((uintptr_t)p);
    }
    if (p) cudaFreeHost(p);
}

// Device address of [p, p + bytes) when the range lies inside one fm_host_alloc
// block of this context (page-locked and mapped: kernels may write it over the
// host link directly), else null.
static void* host_mapped(fm_ctx* ctx, const void* p, size_t bytes) {
    if (!p || ctx->host_allocs.empty()) return nullptr;
    const uintptr_t a = (uintptr_t)p;
    auto it = ctx->host_allocs.upper_bound(a);
    if (it == ctx->host_allocs.begin()) return nullptr;
    --it;
    const uintptr_t base = it->first;
    const size_t size = it->second.first;
    if (a - base > size || bytes > size - (a - base)) return nullptr;
    return (char*)it->second.second + (a - base);
}

static int scene_build(fm_scene* s, const float* xyz, uint64_t n, uint32_t stride, int mem) {
    fm_ctx* ctx = s->ctx;
    const float* d_xyz = xyz;
    if (mem == FM_MEM_HOST) {
        size_t bytes = (size_t)n * stride * sizeof(float);
        if (!grow(ctx->stage[0], bytes)) return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
        FM_CUDA(ctx, cudaMemcpyAsync(ctx->stage[0].p, xyz, bytes, cudaMemcpyHostToDevice, ctx->stream));
        d_xyz = (const float*)ctx->stage[0].p;
    }
    s->n = n;
    s->gen = 0;  // a failed rebuild leaves no valid generation
    int rc = build_grid(ctx, s, d_xyz, stride);
    if (rc != FM_OK) return rc;
    FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    s->gen = ++ctx->gen_counter;
    return FM_OK;
}

int fm_scene_create(fm_ctx* ctx, const float* xyz, uint64_t n, uint32_t stride, float support_radius, int mem,
                    fm_scene** out) {
    if (!ctx || !out) return FM_ERR_INVALID;
    *out = nullptr;
    if (!xyz) return set_err(ctx, FM_ERR_INVALID, "positions are NULL");
    if (n == 0) return set_err(ctx, FM_ERR_INVALID, "scene has no particles");
    if (n >= (1ull << 32)) return set_err(ctx, FM_ERR_INVALID, "more than 2^32 - 1 particles");
    if (stride < 3) return set_err(ctx, FM_ERR_INVALID, "stride must be >= 3 floats");
    if (!(support_radius > 0.0f) || !std::isfinite(support_radius))
        return set_err(ctx, FM_ERR_INVALID, "support radius must be positive and finite");
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    cudaSetDevice(ctx->device);
    fm_scene* s = new (std::nothrow) fm_scene();
    if (!s) return set_err(ctx, FM_ERR_OOM, "host allocation failed");
    s->ctx = ctx;
    s->support = support_radius;
    s->capacity = n;
    if (cudaMalloc(&s->d_pts, n * sizeof(float4)) != cudaSuccess ||
        cudaMalloc(&s->d_cell, n * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&s->d_perm, n * sizeof(uint32_t)) != cudaSuccess) {
        fm_scene_destroy(s);
        return set_err(ctx, FM_ERR_OOM, "particle buffer allocation failed");
    }
    int rc = scene_build(s, xyz, n, stride, mem);
    if (rc != FM_OK) {
        fm_scene_destroy(s);
        return rc;
    }
    ctx->scenes.push_back(s);
    *out = s;
    return FM_OK;
}

int fm_scene_update(fm_scene* s, const float* xyz, uint64_t n, uint32_t stride, int mem) {
    if (!s) return FM_ERR_INVALID;
    fm_ctx* ctx = s->ctx;
    if (!xyz || n == 0) return set_err(ctx, FM_ERR_INVALID, "positions are NULL or empty");
    if (n > s->capacity) return set_err(ctx, FM_ERR_INVALID, "update has more particles than the scene's capacity");
    if (stride < 3) return set_err(ctx, FM_ERR_INVALID, "stride must be >= 3 floats");
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    cudaSetDevice(ctx->device);
    return scene_build(s, xyz, n, stride, mem);
}

int fm_scene_upload(fm_ctx* ctx, const float* xyz, uint64_t n, int32_t stride_floats, float support_radius,
                    fm_scene** out) {
    if (stride_floats < 0) return ctx ? set_err(ctx, FM_ERR_INVALID, "negative stride") : FM_ERR_INVALID;
    return fm_scene_create(ctx, xyz, n, (uint32_t)stride_floats, support_radius, FM_MEM_HOST, out);
}

void fm_scene_destroy(fm_scene* s) {
    if (!s) return;
    fm_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);  // a bound table build of the scene
    for (size_t i = 0; i < ctx->scenes.size(); ++i)
        if (ctx->scenes[i] == s) {
            ctx->scenes.erase(ctx->scenes.begin() + i);
            break;
        }
    scene_free(s);
}

int fm_scene_grid(const fm_scene* s, fm_grid_info* out) {
    if (!s || !out) return FM_ERR_INVALID;
    for (int a = 0; a < 3; ++a) {
        out->min[a] = s->min[a];
        out->max[a] = s->max[a];
        out->dims[a] = s->dims[a];
    }
    out->cell_width = 1.0f * s->support;
    out->inv_cell_width = s->inv;
    out->pad = 0;
    out->n_particles = s->n;
    out->n_cells = s->ncells;
    return FM_OK;
}

int fm_scene_download(const fm_scene* s, uint32_t* cell, uint32_t* sorted_index, uint32_t* cell_start,
                      float* sorted_xyzw) {
    if (!s) return FM_ERR_INVALID;
    fm_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (cell) FM_CUDA(ctx, cudaMemcpy(cell, s->d_cell, s->n * 4, cudaMemcpyDeviceToHost));
    if (sorted_index) FM_CUDA(ctx, cudaMemcpy(sorted_index, s->d_perm, s->n * 4, cudaMemcpyDeviceToHost));
    // every 8th sub-cell start is a cell start (the last one is n)
    if (cell_start)
        FM_CUDA(ctx, cudaMemcpy2D(cell_start, 4, s->d_sub, 32, 4, s->ncells + 1, cudaMemcpyDeviceToHost));
    if (sorted_xyzw) FM_CUDA(ctx, cudaMemcpy(sorted_xyzw, s->d_pts, s->n * 16, cudaMemcpyDeviceToHost));
    return FM_OK;
}

int fm_splat_depth(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, float* depth, int mem, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!s || !depth) return set_err(ctx, FM_ERR_INVALID, "scene or depth buffer is NULL");
    int rc = check_camera(ctx, cam, true);
    if (rc) return rc;
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    size_t bytes = (size_t)cam->width * cam->height * sizeof(float);
    float* d = depth;
    if (mem == FM_MEM_HOST) {
        if (!grow(ctx->stage[1], bytes)) return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
        d = (float*)ctx->stage[1].p;
    }
    rc = launch_splat(ctx, s, cam, d, st);
    if (rc) return rc;
    if (mem == FM_MEM_HOST) {
        FM_CUDA(ctx, cudaMemcpyAsync(depth, d, bytes, cudaMemcpyDeviceToHost, st));
        FM_CUDA(ctx, cudaStreamSynchronize(st));
    }
    return FM_OK;
}

int fm_density(fm_ctx* ctx, const fm_scene* s, const float* xyz, uint64_t n, uint32_t stride, float* out, int mem,
               void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!s || (n && (!xyz || !out))) return set_err(ctx, FM_ERR_INVALID, "NULL argument");
    if (stride < 3) return set_err(ctx, FM_ERR_INVALID, "stride must be >= 3 floats");
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    if (n == 0) return FM_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    if (mem == FM_MEM_DEVICE) return launch_density(ctx, s, xyz, n, stride, out, st);
    const size_t in_bytes = (size_t)n * stride * sizeof(float), out_bytes = (size_t)n * sizeof(float);
    if (!grow(ctx->stage[0], in_bytes) || !grow(ctx->stage[1], out_bytes))
        return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
    FM_CUDA(ctx, cudaMemcpyAsync(ctx->stage[0].p, xyz, in_bytes, cudaMemcpyHostToDevice, st));
    int rc = launch_density(ctx, s, (const float*)ctx->stage[0].p, n, stride, (float*)ctx->stage[1].p, st);
    if (rc) return rc;
    FM_CUDA(ctx, cudaMemcpyAsync(out, ctx->stage[1].p, out_bytes, cudaMemcpyDeviceToHost, st));
    FM_CUDA(ctx, cudaStreamSynchronize(st));
    return FM_OK;
}

int fm_set_anisotropy(fm_ctx* ctx, const fm_aniso_params* p) {
    if (!ctx) return FM_ERR_INVALID;
    if (!p) {
        ctx->aniso = fm_aniso_params{2.0f, 0.5f, 2.0f, 2000.0f, 1, 0};
        return FM_OK;
    }
    if (!(p->radius_mult >= 1.0f && p->radius_mult <= 2.0f))
        return set_err(ctx, FM_ERR_INVALID, "radius_mult must be in [1, 2] (the march walks 5x5x5 cells)");
    if (!(p->k_n > 0.0f) || !(p->k_r > 0.0f) || !(p->k_s > 0.0f) || !std::isfinite(p->k_n) || !std::isfinite(p->k_r) ||
        !std::isfinite(p->k_s))
        return set_err(ctx, FM_ERR_INVALID, "k_n, k_r and k_s must be positive and finite");
    if (p->n_eps < 0 || p->reserved != 0) return set_err(ctx, FM_ERR_INVALID, "n_eps must be >= 0, reserved 0");
    ctx->aniso = *p;
    return FM_OK;
}

int fm_set_stats(fm_ctx* ctx, int enable) {
    if (!ctx) return FM_ERR_INVALID;
    ctx->stats_enabled = enable ? 1 : 0;
    return FM_OK;
}

int fm_march_stats_get(fm_ctx* ctx, fm_march_stats* out) {
    if (!ctx || !out) return FM_ERR_INVALID;
    cudaSetDevice(ctx->device);
    FM_CUDA(ctx, cudaDeviceSynchronize());
    unsigned long long h[fm::kStatSlots];
    FM_CUDA(ctx, cudaMemcpy(h, ctx->d_stats, sizeof(h), cudaMemcpyDeviceToHost));
    out->rays = h[0];
    out->started = h[1];
    out->hits = h[2];
    out->evals = h[3];
    out->candidates = h[4];
    out->skipped = h[5];
    out->tested = h[6];
    out->streamed = h[7];
    out->deferred = h[8];
    out->proposed = h[9];
    out->fallbacks = h[10];
    out->regrouped = h[11];
    return FM_OK;
}

int fm_march(fm_ctx* ctx, const fm_scene* s, const fm_camera* cam, const fm_march_params* p, const fm_frame_out* out,
             int mem, void* stream) {
    if (!ctx) return FM_ERR_INVALID;
    if (!s || !out) return set_err(ctx, FM_ERR_INVALID, "scene or output description is NULL");
    int rc = check_params(ctx, p);
    if (rc) return rc;
    const bool external = (p->flags & FM_MARCH_EXTERNAL_DEPTH) != 0;
    rc = check_camera(ctx, cam, !external);
    if (rc) return rc;
    if (mem != FM_MEM_HOST && mem != FM_MEM_DEVICE) return set_err(ctx, FM_ERR_INVALID, "unknown memory kind");
    if (external && !out->start_depth)
        return set_err(ctx, FM_ERR_INVALID, "FM_MARCH_EXTERNAL_DEPTH needs fm_frame_out.start_depth");
    cudaSetDevice(ctx->device);
    cudaStream_t st = pick(ctx, stream);
    const size_t npx = (size_t)cam->width * cam->height;
    fm_scene* sm = const_cast<fm_scene*>(s);
    // the grid itself was built synchronously; skip tables are built once per
    // scene (the bound table again for a higher iso).  A bound table this
    // march needs is built on the side stream while the splat runs here.
    const bool overlap = p->skip_mode == FM_SKIP_EXACT && !external && bound_stale(sm, p->iso_density);
    if (p->skip_mode == FM_SKIP_EXACT && !overlap && (rc = ensure_bound(ctx, sm, st, p->iso_density)) != FM_OK)
        return rc;

    if (p->skip_mode == FM_SKIP_REFERENCE && (rc = ensure_flags(ctx, sm, st)) != FM_OK) return rc;
    MarchOutDev o{};
    const bool host = mem == FM_MEM_HOST;
    // ray-start depth
    float* z = nullptr;
    if (external) {
        if (host) {
            if (!grow(ctx->stage[1], npx * 4)) return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
            z = (float*)ctx->stage[1].p;
            FM_CUDA(ctx, cudaMemcpyAsync(z, out->start_depth, npx * 4, cudaMemcpyHostToDevice, st));
        } else {
            z = out->start_depth;
        }
    } else {
        if (!host && out->start_depth) {
            z = out->start_depth;
        } else {
            if (!grow(ctx->stage[1], npx * 4)) return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
            z = (float*)ctx->stage[1].p;
        }
        if (overlap) {
            FM_CUDA(ctx, cudaEventRecord(ctx->ev_fork, st));
            FM_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
            if ((rc = ensure_bound(ctx, sm, ctx->side, p->iso_density)) != FM_OK) return rc;
            FM_CUDA(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
        }
        rc = launch_splat(ctx, s, cam, z, st);
        // whatever the splat returned, work queued on st after this point sees the table
        if (overlap) FM_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_join, 0));
        if (rc) return rc;
    }
    o.start_depth = z;
    o.ivl = nullptr;
    if (p->flags & FM_MARCH_PROPOSAL) {
        if (p->skip_mode == FM_SKIP_REFERENCE)
            return set_err(ctx, FM_ERR_INVALID, "FM_MARCH_PROPOSAL marches the plain sample lattice: skip mode must be off or exact");
        if (!ctx->proposal) return set_err(ctx, FM_ERR_INVALID, "FM_MARCH_PROPOSAL needs a proposal (fm_set_proposal)");
        if (!grow(ctx->prop_ivl, npx * sizeof(int2))) return set_err(ctx, FM_ERR_OOM, "interval buffer allocation failed");
        rc = launch_propose(ctx, sm, cam, p, ctx->proposal, z, (int2*)ctx->prop_ivl.p, nullptr, st);
        if (rc) return rc;
        o.ivl = (const int2*)ctx->prop_ivl.p;
    }
    float* user[4] = {out->position, out->normal, out->depth, out->colour};
    const size_t per[4] = {16, 16, 4, 16};
    void* dev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool direct[4] = {false, false, false, false};
    for (int i = 0; i < 4; ++i) {
        if (!user[i]) continue;
        // outputs in fm_host_alloc memory: the march writes them over the host link
        // itself (each pixel once, coalesced), no copy afterwards
        if (host && (dev[i] = host_mapped(ctx, user[i], npx * per[i])) != nullptr) {
            direct[i] = true;
            continue;
        }
        if (host) {
            if (!grow(ctx->stage[2 + i], npx * per[i])) return set_err(ctx, FM_ERR_OOM, "staging allocation failed");
            dev[i] = ctx->stage[2 + i].p;
        } else {
            dev[i] = user[i];
        }
    }
    o.pos = (float4*)dev[0];
    o.nrm = (float4*)dev[1];
    o.depth = (float*)dev[2];
    o.col = (float4*)dev[3];
    const bool judge = (p->flags & FM_MARCH_PROPOSAL) && ctx->judge_stride > 0;
    if (judge && !o.depth) {  // the judge compares hit distances: the learned march writes them here
        if (!grow_buf(ctx->judge_test, npx * 4)) return set_err(ctx, FM_ERR_OOM, "judge buffer allocation failed");
        o.depth = (float*)ctx->judge_test.p;
    }
    if (ctx->stats_enabled) FM_CUDA(ctx, cudaMemsetAsync(ctx->d_stats, 0, fm::kStatSlots * sizeof(unsigned long long), st));
    if (judge) {
        // the judge's sample march runs on the side stream next to the learned march
        FM_CUDA(ctx, cudaEventRecord(ctx->ev_jfork, st));
        FM_CUDA(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_jfork, 0));
        rc = judge_start(ctx, sm, cam, p, z, ctx->side);
        // whatever it returned, st waits for what reached the side stream
        FM_CUDA(ctx, cudaEventRecord(ctx->ev_jjoin, ctx->side));
        if (rc) {
            FM_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_jjoin, 0));
            return rc;
        }
    }
    if (p->flags & FM_MARCH_ANISOTROPIC) rc = launch_march_aniso(ctx, s, cam, p, &ctx->aniso, o, st);
    else rc = launch_march(ctx, s, cam, p, o, st);
    if (judge) {
        FM_CUDA(ctx, cudaStreamWaitEvent(st, ctx->ev_jjoin, 0));
        if (!rc) rc = judge_finish(ctx, o.depth, npx, st);
    }
    if (rc) return rc;
    if (host) {
        for (int i = 0; i < 4; ++i)
            if (user[i] && !direct[i])
                FM_CUDA(ctx, cudaMemcpyAsync(user[i], dev[i], npx * per[i], cudaMemcpyDeviceToHost, st));
        if (out->start_depth && !external)
            FM_CUDA(ctx, cudaMemcpyAsync(out->start_depth, z, npx * 4, cudaMemcpyDeviceToHost, st));
        // every host buffer in fm_host_alloc memory: nothing has to wait here, the
        // call is asynchronous as with device buffers (fm_query / fm_sync)
        bool all_pinned = true;
        for (int i = 0; i < 4; ++i) all_pinned = all_pinned && (!user[i] || direct[i]);
        if (out->start_depth) all_pinned = all_pinned && host_mapped(ctx, out->start_depth, npx * 4) != nullptr;
        if (all_pinned) return FM_OK;
        unsigned int* hs = (unsigned int*)ctx->h_pinned_small;
        FM_CUDA(ctx, cudaMemcpyAsync(hs, ctx->d_status, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        FM_CUDA(ctx, cudaStreamSynchronize(st));
        if (hs[0] != 0) {
            unsigned int code = hs[0];
            cudaMemset(ctx->d_status, 0, sizeof(unsigned int));
            return set_err(ctx, FM_ERR_DEVICE, "march kernel status word set: " + std::to_string(code));
        }
    }
    return FM_OK;
}

}  // extern "C"
