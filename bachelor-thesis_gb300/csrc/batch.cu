// batch.cu -- many views of many scenes in one launch per pass, under a CUDA graph.
//
// The reference renders one view per RayMarcher::Start (RayMarcher.cpp:102-112)
// with a thread pool over the pixels of that view (ThreadPool.cpp:5-55).  A
// batch instead lays the views of any number of scenes (uneven particle
// counts, resolutions, march settings) end to end: every pass of the frame
// (depth fill, sampled splat, tile maxima, cull, survivor splat, march, long
// rays) is one launch whose persistent warps walk the units of all views, and
// a view is found from a unit by a binary search over per-view prefix sums.
// The seven launches and the counter reset are captured once into a CUDA
// graph; a frame is one cudaGraphLaunch.
//
// fm_batch_autotune times the batch under candidate work splits (tile shape,
// tiles per claim, iterations before deferral) and keeps the fastest; results
// do not depend on the split.

#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "fm_internal.cuh"

struct fm_batch {
    fm_ctx* ctx = nullptr;
    std::vector<fm_view> views;
    std::vector<uint64_t> gens;  // scene generations the arguments were built from
    fm::TileConfig cfg;
    // device buffers
    fm::DevBuf margs, tile_pfx, sviews, pfx64, pfx_tiles, depth, hiz, list, counters, longq;
    fm::DevBuf longq2, rg_keys, rg_tmp, rg_order;  // regrouped second pass
    // learned proposal of the views with FM_MARCH_PROPOSAL: the weights (a copy),
    // per-view blocks, tile and low-resolution prefixes, low-resolution depths,
    // intervals of every pixel
    fm::DevBuf pw, pb, pviews, ptile_pfx, plow_pfx, plow, pivl, pblk_pfx;
    float pmargins[3] = {0.0f, 0.0f, 0.0f};  // margin_lo, margin_hi, min_near of the copied proposal
    // anisotropic views: the context's kernel settings at creation, per-view
    // blocks, 32-pixel chunk prefixes, the chunk total
    fm_aniso_params aniso{};
    fm::DevBuf aviews, apfx;
    uint32_t achunks = 0;
    fm::ProposeBatchDev pbatch{};
    uint32_t q_cap = 0;
    fm::MarchArgs launch{};  // launch-wide march arguments
    fm::SplatBatch sb{};
    uint64_t pixels = 0, particles = 0, tiles = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int nodes = 0;
};

namespace fm {
namespace {

constexpr int kMaxViews = 1 << 16;

void drop_graph(fm_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->nodes = 0;
}

void free_batch(fm_batch* b) {
    // a graph of this batch may still run on any stream
    cudaDeviceSynchronize();
    drop_graph(b);
    DevBuf* bufs[] = {&b->margs,  &b->tile_pfx, &b->sviews,  &b->pfx64,   &b->pfx_tiles, &b->depth,
                      &b->hiz,    &b->list,     &b->counters, &b->longq,  &b->longq2,    &b->rg_keys,
                      &b->rg_tmp, &b->rg_order, &b->pw,       &b->pb,     &b->pviews,    &b->ptile_pfx,
                      &b->plow_pfx, &b->plow,   &b->pivl,     &b->aviews,   &b->apfx,      &b->pblk_pfx};
    for (DevBuf* d : bufs) cudaFree(d->p);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    delete b;
}

int check_config(fm_ctx* ctx, const fm_tile_config* c, TileConfig* out) {
    if (!c) return set_err(ctx, FM_ERR_INVALID, "tile config is NULL");
    int lg = -1;
    for (int i = 0; i <= 5; ++i)
        if (c->tile_width == (1 << i)) lg = i;
    if (lg < 0) return set_err(ctx, FM_ERR_INVALID, "tile_width must be 1, 2, 4, 8, 16 or 32");
    if (c->tiles_per_claim < 1 || c->tiles_per_claim > 16)
        return set_err(ctx, FM_ERR_INVALID, "tiles_per_claim must be in [1, 16]");
    if (c->defer_iters < 0 || c->defer_iters > 4096)
        return set_err(ctx, FM_ERR_INVALID, "defer_iters must be in [0, 4096]");
    if (c->long_queue < 0) return set_err(ctx, FM_ERR_INVALID, "long_queue must be >= 0");
    if (c->defer_lanes < 0 || c->defer_lanes > 31) return set_err(ctx, FM_ERR_INVALID, "defer_lanes must be in [0, 31]");
    if (c->regroup_iters < 0 || c->regroup_iters > 4096)
        return set_err(ctx, FM_ERR_INVALID, "regroup_iters must be in [0, 4096]");
    out->tw_log2 = lg;
    out->claim = c->tiles_per_claim;
    out->cap = c->defer_iters;
    out->qlimit = (uint32_t)c->long_queue;
    out->lanes = c->defer_lanes;
    out->cap2 = c->regroup_iters;
    return FM_OK;
}

fm_tile_config to_public(const TileConfig& c) {
    fm_tile_config o{};
    o.tile_width = 1 << c.tw_log2;
    o.tiles_per_claim = c.claim;
    o.defer_iters = c.cap;
    o.long_queue = (int32_t)c.qlimit;
    o.defer_lanes = c.lanes;
    o.regroup_iters = c.cap2;
    return o;
}

// Sizes, skip tables, buffers and argument blocks for the current scenes and
// work split.  Synchronous.
int prepare(fm_batch* b) {
    fm_ctx* ctx = b->ctx;
    const int n = (int)b->views.size();
    // a run of this batch may still be reading the argument blocks
    FM_CUDA(ctx, cudaDeviceSynchronize());
    // skip tables of the scenes, built once on the context stream
    for (const fm_view& v : b->views) {
        fm_scene* s = const_cast<fm_scene*>(v.scene);
        int rc = FM_OK;
        if (v.params.skip_mode == FM_SKIP_EXACT) rc = ensure_bound(ctx, s, ctx->stream, v.params.iso_density);
        if (!rc && v.params.skip_mode == FM_SKIP_REFERENCE) rc = ensure_flags(ctx, s, ctx->stream);
        if (!rc && (v.params.flags & FM_MARCH_PROPOSAL)) rc = ensure_occupancy(ctx, s, ctx->stream);
        if (rc) return rc;
    }
    FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // prefix sums
    std::vector<uint64_t> px(n + 1, 0), smp(n + 1, 0), pn(n + 1, 0);
    std::vector<uint32_t> ht(n + 1, 0), tp(n + 1, 0), ap(n + 1, 0);
    const int tw = 1 << b->cfg.tw_log2, th = 32 >> b->cfg.tw_log2;
    for (int i = 0; i < n; ++i) {
        const fm_view& v = b->views[i];
        const uint64_t w = (uint64_t)v.camera.width, h = (uint64_t)v.camera.height;
        px[i + 1] = px[i] + w * h;
        smp[i + 1] = smp[i] + (v.scene->n + kSplatSample - 1) / kSplatSample;
        pn[i + 1] = pn[i] + v.scene->n;
        const uint64_t hz = ((w + kSplatHizTile - 1) / kSplatHizTile) * ((h + kSplatHizTile - 1) / kSplatHizTile);
        // anisotropic views are marched by their own launch in 32-pixel chunks
        const bool an = (v.params.flags & FM_MARCH_ANISOTROPIC) != 0;
        const uint64_t tl = an ? 0 : ((w + tw - 1) / tw) * ((h + th - 1) / th);
        const uint64_t ch = an ? (w * h + 31) / 32 : 0;
        if ((uint64_t)ht[i] + hz >= (1ull << 32) || (uint64_t)tp[i] + tl >= (1ull << 31) ||
            (uint64_t)ap[i] + ch >= (1ull << 31))
            return set_err(ctx, FM_ERR_INVALID, "batch has too many tiles");
        ht[i + 1] = ht[i] + (uint32_t)hz;
        tp[i + 1] = tp[i] + (uint32_t)tl;
        ap[i + 1] = ap[i] + (uint32_t)ch;
    }
    if (pn[n] >= (1ull << 32)) return set_err(ctx, FM_ERR_INVALID, "batch has 2^32 or more particles");
    const uint64_t entries = long_queue_entries(px[n], b->cfg.qlimit);
    if (entries >= (1ull << 32)) return set_err(ctx, FM_ERR_INVALID, "batch has too many pixels");
    b->pixels = px[n];
    b->particles = pn[n];
    b->tiles = tp[n];
    // buffers (grown, never shrunk)
    FM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!grow_buf(b->margs, sizeof(MarchArgs) * n) || !grow_buf(b->tile_pfx, 4ull * (n + 1)) ||
        !grow_buf(b->sviews, sizeof(SplatView) * n) || !grow_buf(b->pfx64, 8ull * 3 * (n + 1)) ||
        !grow_buf(b->pfx_tiles, 4ull * (n + 1)) || !grow_buf(b->depth, 4ull * std::max<uint64_t>(px[n], 1)) ||
        !grow_buf(b->hiz, 4ull * std::max<uint32_t>(ht[n], 1)) ||
        !grow_buf(b->list, 4ull * std::max<uint64_t>(pn[n], 1)) || !grow_buf(b->counters, 128) ||
        !grow_buf(b->longq, 64ull * entries) || !grow_buf(b->aviews, aniso_view_bytes() * n) ||
        !grow_buf(b->apfx, 4ull * (n + 1)))
        return set_err(ctx, FM_ERR_OOM, "batch buffer allocation failed");
    const bool regroup = b->cfg.cap2 > 0;
    const uint64_t nkeys = (uint64_t)tp[n] + 1;
    if (regroup && (!grow_buf(b->longq2, 64ull * entries) || !grow_buf(b->rg_order, 4ull * entries) ||
                    !grow_buf(b->rg_keys, 4ull * nkeys) || !grow_buf(b->rg_tmp, 4ull * scan_words(nkeys))))
        return set_err(ctx, FM_ERR_OOM, "batch buffer allocation failed");
    b->q_cap = (uint32_t)entries;
    unsigned int* cnt = (unsigned int*)b->counters.p;
    // learned proposal: blocks for the views that use it
    std::vector<int> pv_idx;
    for (int i = 0; i < n; ++i)
        if (b->views[i].params.flags & FM_MARCH_PROPOSAL) pv_idx.push_back(i);
    const int np = (int)pv_idx.size();
    std::vector<uint64_t> ptp(np + 1, 0), plp(np + 1, 0), pbp(np + 1, 0);
    for (int k = 0; k < np; ++k) {
        const fm_view& v = b->views[pv_idx[k]];
        const uint64_t npx = (uint64_t)v.camera.width * v.camera.height;
        ptp[k + 1] = ptp[k] + (npx + 127) / 128;
        plp[k + 1] = plp[k] + propose_low_pixels(&v.camera);
        pbp[k + 1] = pbp[k] + propose_view_blocks(&v.camera);
    }
    if (np > 0) {
        if (!grow_buf(b->pviews, propose_view_bytes() * np) || !grow_buf(b->ptile_pfx, 8ull * (np + 1)) ||
            !grow_buf(b->plow_pfx, 8ull * (np + 1)) || !grow_buf(b->pblk_pfx, 8ull * (np + 1)) ||
            !grow_buf(b->plow, 4ull * std::max<uint64_t>(plp[np], 1)) ||
            !grow_buf(b->pivl, 8ull * std::max<uint64_t>(px[n], 1)))
            return set_err(ctx, FM_ERR_OOM, "batch buffer allocation failed");
    }
    // march arguments: per view, with the launch-wide fields in every block
    std::vector<MarchArgs> ma(n);
    std::vector<SplatView> sv(n);
    float* depth = (float*)b->depth.p;
    for (int i = 0; i < n; ++i) {
        const fm_view& v = b->views[i];
        float* z = v.out.start_depth ? v.out.start_depth : depth + px[i];
        MarchOutDev o{};
        o.ivl = (v.params.flags & FM_MARCH_PROPOSAL) ? (const int2*)b->pivl.p + px[i] : nullptr;
        o.pos = (float4*)v.out.position;
        o.nrm = (float4*)v.out.normal;
        o.depth = v.out.depth;
        o.col = (float4*)v.out.colour;
        o.start_depth = z;
        // a batch's long pass takes the deferred rays of every view: by default
        // deferral after 24 sums (the 128-view 4K batch of 4M-particle scenes,
        // ms per launch: 3516 after 12 sums, the single-view default; 3029
        // after 15, 2917 after 20, 2893 after 24, 2879 after 32; the 146-view
        // batch's autotune picks 20-24)
        TileConfig vc = b->cfg;
        if (vc.cap == 0) vc.cap = 24;
        MarchArgs a = march_view_args(v.scene, &v.camera, &v.params, o, vc);
        a.tile_counter = cnt;
        a.q_tail = cnt + 1;
        a.q_head = cnt + 2;
        a.longq = (float4*)b->longq.p;
        a.q_cap = b->q_cap;
        a.status = ctx->d_status;
        a.stats = nullptr;
        a.grp_counter = cnt + 4;
        a.q2_tail = cnt + 5;
        a.q2_head = cnt + 6;
        if (regroup) {
            a.longq2 = (float4*)b->longq2.p;
            a.order = (uint32_t*)b->rg_order.p;
            a.keys = (uint32_t*)b->rg_keys.p;
            a.scan_tmp = (uint32_t*)b->rg_tmp.p;
        }
        ma[i] = a;
        SplatView s{};
        s.a = splat_args(v.scene, &v.camera);
        s.a.hiz = (const float*)b->hiz.p + ht[i];
        s.pts = v.scene->d_pts;
        s.n = v.scene->n;
        s.depth = (uint32_t*)z;
        sv[i] = s;
    }
    b->launch = ma[0];
    b->launch.ntiles = (int)tp[n];
    // the learned instantiation runs when any view has a proposal (views without one march fully)
    b->launch.ivl = np > 0 ? (const int2*)b->pivl.p : nullptr;
    if (np > 0) {
        std::vector<uint8_t> blocks(propose_view_bytes() * np);
        for (int k = 0; k < np; ++k) {
            const int i = pv_idx[k];
            const fm_view& v = b->views[i];
            propose_view(v.scene, &v.camera, &v.params, b->pmargins, ma[i].zbuf, (float*)b->plow.p + plp[k],
                         (int2*)b->pivl.p + px[i], blocks.data() + propose_view_bytes() * k);
        }
        FM_CUDA(ctx, cudaMemcpy(b->pviews.p, blocks.data(), blocks.size(), cudaMemcpyHostToDevice));
        FM_CUDA(ctx, cudaMemcpy(b->ptile_pfx.p, ptp.data(), 8ull * (np + 1), cudaMemcpyHostToDevice));
        FM_CUDA(ctx, cudaMemcpy(b->plow_pfx.p, plp.data(), 8ull * (np + 1), cudaMemcpyHostToDevice));
        FM_CUDA(ctx, cudaMemcpy(b->pblk_pfx.p, pbp.data(), 8ull * (np + 1), cudaMemcpyHostToDevice));
    }
    b->pbatch = ProposeBatchDev{b->pviews.p, (const uint64_t*)b->ptile_pfx.p, (const uint64_t*)b->plow_pfx.p, np,
                                ptp[np], plp[np], (const uint64_t*)b->pblk_pfx.p, pbp[np], b->pw.p,
                                (const float*)b->pb.p};
    {
        std::vector<uint8_t> blocks(aniso_view_bytes() * n, 0);
        for (int i = 0; i < n; ++i)
            if (b->views[i].params.flags & FM_MARCH_ANISOTROPIC)
                aniso_view(b->views[i].scene, &b->aniso, blocks.data() + aniso_view_bytes() * i);
        FM_CUDA(ctx, cudaMemcpy(b->aviews.p, blocks.data(), blocks.size(), cudaMemcpyHostToDevice));
        FM_CUDA(ctx, cudaMemcpy(b->apfx.p, ap.data(), 4ull * (n + 1), cudaMemcpyHostToDevice));
        b->achunks = ap[n];
    }
    b->gens.resize(n);
    for (int i = 0; i < n; ++i) b->gens[i] = b->views[i].scene->gen;
    FM_CUDA(ctx, cudaMemcpy(b->margs.p, ma.data(), sizeof(MarchArgs) * n, cudaMemcpyHostToDevice));
    FM_CUDA(ctx, cudaMemcpy(b->tile_pfx.p, tp.data(), 4ull * (n + 1), cudaMemcpyHostToDevice));
    FM_CUDA(ctx, cudaMemcpy(b->sviews.p, sv.data(), sizeof(SplatView) * n, cudaMemcpyHostToDevice));
    uint64_t* p64 = (uint64_t*)b->pfx64.p;
    FM_CUDA(ctx, cudaMemcpy(p64, px.data(), 8ull * (n + 1), cudaMemcpyHostToDevice));
    FM_CUDA(ctx, cudaMemcpy(p64 + (n + 1), smp.data(), 8ull * (n + 1), cudaMemcpyHostToDevice));
    FM_CUDA(ctx, cudaMemcpy(p64 + 2 * (n + 1), pn.data(), 8ull * (n + 1), cudaMemcpyHostToDevice));
    FM_CUDA(ctx, cudaMemcpy(b->pfx_tiles.p, ht.data(), 4ull * (n + 1), cudaMemcpyHostToDevice));
    SplatBatch& s = b->sb;
    s.views = (const SplatView*)b->sviews.p;
    s.nviews = n;
    s.pfx_px = p64;
    s.pfx_sample = p64 + (n + 1);
    s.pfx_n = p64 + 2 * (n + 1);
    s.pfx_tiles = (const uint32_t*)b->pfx_tiles.p;
    s.hiz = (float*)b->hiz.p;
    s.list = (uint32_t*)b->list.p;
    s.count = cnt + 3;
    s.tot_px = px[n];
    s.tot_sample = smp[n];
    s.tot_n = pn[n];
    s.tot_tiles = ht[n];
    return FM_OK;
}

// The frame's work on `st`: counter reset, depth pass, march.
int enqueue(fm_batch* b, cudaStream_t st, bool stats) {
    fm_ctx* ctx = b->ctx;
    FM_CUDA(ctx, cudaMemsetAsync(b->counters.p, 0, 8 * sizeof(unsigned int), st));
    int rc = launch_splat_batch(ctx, b->sb, st);
    if (rc) return rc;
    if (b->pbatch.nviews > 0 && (rc = launch_propose_batch(ctx, b->pbatch, st)) != FM_OK) return rc;
    MarchArgs a = b->launch;
    a.stats = stats ? ctx->d_stats : nullptr;
    const int n = (int)b->views.size();
    if (a.ntiles > 0 &&
        (rc = launch_march_kernels(ctx, a, (const MarchArgs*)b->margs.p, (const uint32_t*)b->tile_pfx.p, n, st)))
        return rc;
    if (b->achunks == 0) return FM_OK;
    a.tile_counter = (unsigned int*)b->counters.p + 7;
    return launch_march_aniso_batch(ctx, a, (const MarchArgs*)b->margs.p, b->aviews.p, (const uint32_t*)b->apfx.p, n,
                                    b->achunks, st);
}

int capture(fm_batch* b) {
    fm_ctx* ctx = b->ctx;
    drop_graph(b);
    FM_CUDA(ctx, cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue(b, b->cap_stream, false);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaStreamEndCapture");
    b->graph = g;
    FM_CUDA(ctx, cudaGraphInstantiate(&b->exec, g, 0));
    size_t nn = 0;
    FM_CUDA(ctx, cudaGraphGetNodes(g, nullptr, &nn));
    b->nodes = (int)nn;
    return FM_OK;
}

}  // namespace

void destroy_batches(fm_ctx* ctx) {
    for (fm_batch* b : ctx->batches) free_batch(b);
    ctx->batches.clear();
}

}  // namespace fm

using namespace fm;

extern "C" {

int fm_set_tile_config(fm_ctx* ctx, const fm_tile_config* cfg) {
    if (!ctx) return FM_ERR_INVALID;
    TileConfig t;
    const int rc = check_config(ctx, cfg, &t);
    if (rc) return rc;
    ctx->tile = t;
    return FM_OK;
}

int fm_get_tile_config(const fm_ctx* ctx, fm_tile_config* out) {
    if (!ctx || !out) return FM_ERR_INVALID;
    *out = to_public(ctx->tile);
    return FM_OK;
}

int fm_batch_create(fm_ctx* ctx, const fm_view* views, int32_t n_views, const fm_tile_config* cfg, fm_batch** out) {
    if (!ctx) return FM_ERR_INVALID;
    if (!out) return set_err(ctx, FM_ERR_INVALID, "output handle pointer is NULL");
    *out = nullptr;
    if (!views || n_views < 1 || n_views > kMaxViews)
        return set_err(ctx, FM_ERR_INVALID, "a batch needs 1 to 65536 views");
    TileConfig t = ctx->tile;
    if (cfg) {
        const int rc = check_config(ctx, cfg, &t);
        if (rc) return rc;
    }
    for (int i = 0; i < n_views; ++i) {
        const fm_view& v = views[i];
        if (!v.scene || std::find(ctx->scenes.begin(), ctx->scenes.end(), v.scene) == ctx->scenes.end())
            return set_err(ctx, FM_ERR_INVALID, "view scene is NULL or not a live scene of this context");
        int rc = check_params(ctx, &v.params);
        if (rc) return rc;
        if (v.params.flags & FM_MARCH_EXTERNAL_DEPTH)
            return set_err(ctx, FM_ERR_INVALID, "batched views are splatted: FM_MARCH_EXTERNAL_DEPTH is not allowed");
        if ((v.params.flags & FM_MARCH_PROPOSAL) && !ctx->proposal)
            return set_err(ctx, FM_ERR_INVALID, "FM_MARCH_PROPOSAL needs a proposal (fm_set_proposal)");
        if ((v.params.flags & FM_MARCH_PROPOSAL) && v.params.skip_mode == FM_SKIP_REFERENCE)
            return set_err(ctx, FM_ERR_INVALID, "FM_MARCH_PROPOSAL marches the plain sample lattice: skip mode must be off or exact");
        rc = check_camera(ctx, &v.camera, true);
        if (rc) return rc;
        if (v.scene->n == 0) return set_err(ctx, FM_ERR_INVALID, "view scene has no particles");
    }
    cudaSetDevice(ctx->device);
    fm_batch* b = new (std::nothrow) fm_batch();
    if (!b) return set_err(ctx, FM_ERR_OOM, "batch allocation failed");
    b->ctx = ctx;
    b->views.assign(views, views + n_views);
    b->cfg = t;
    b->aniso = ctx->aniso;
    if (cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        free_batch(b);
        return set_err(ctx, FM_ERR_CUDA, "stream creation failed");
    }
    int rc = FM_OK;
    // the batch keeps its own copy of the context's proposal: later fm_set_proposal or
    // fm_proposal_destroy calls do not change it
    bool learned = false;
    for (const fm_view& v : b->views) learned |= (v.params.flags & FM_MARCH_PROPOSAL) != 0;
    if (learned) {
        rc = proposal_weights(ctx, ctx->proposal, b->pw, b->pb, b->pmargins, ctx->stream);
        if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            rc = set_err(ctx, FM_ERR_CUDA, "proposal copy failed");
    }
    if (!rc) rc = prepare(b);
    if (!rc) rc = capture(b);
    if (rc) {
        free_batch(b);
        return rc;
    }
    ctx->batches.push_back(b);
    *out = b;
    return FM_OK;
}

int fm_batch_run(fm_batch* b, void* stream) {
    if (!b) return FM_ERR_INVALID;
    fm_ctx* ctx = b->ctx;
    // every scene must still be alive and unchanged since the arguments were built
    for (size_t i = 0; i < b->views.size(); ++i) {
        const fm_scene* s = b->views[i].scene;
        if (std::find(ctx->scenes.begin(), ctx->scenes.end(), s) == ctx->scenes.end() || s->gen != b->gens[i])
            return set_err(ctx, FM_ERR_INVALID, "a scene of the batch was destroyed or updated: fm_batch_refresh first");
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (ctx->stats_enabled) {
        FM_CUDA(ctx, cudaMemsetAsync(ctx->d_stats, 0, kStatSlots * sizeof(unsigned long long), st));
        return enqueue(b, st, true);
    }
    if (!b->exec) return set_err(ctx, FM_ERR_INVALID, "batch has no graph");
    FM_CUDA(ctx, cudaGraphLaunch(b->exec, st));
    return FM_OK;
}

int fm_batch_refresh(fm_batch* b) {
    if (!b) return FM_ERR_INVALID;
    fm_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    for (const fm_view& v : b->views) {
        if (std::find(ctx->scenes.begin(), ctx->scenes.end(), v.scene) == ctx->scenes.end())
            return set_err(ctx, FM_ERR_INVALID, "a scene of the batch was destroyed");
        if (v.scene->gen == 0) return set_err(ctx, FM_ERR_INVALID, "a scene of the batch has no valid grid");
    }
    int rc = prepare(b);
    if (!rc) rc = capture(b);
    return rc;
}

int fm_batch_autotune(fm_batch* b, const fm_tile_config* cands, int32_t n_cands, int32_t reps, fm_tile_config* best,
                      float* best_ms) {
    if (!b) return FM_ERR_INVALID;
    fm_ctx* ctx = b->ctx;
    if (reps < 1 || reps > 100) return set_err(ctx, FM_ERR_INVALID, "reps must be in [1, 100]");
    if (cands && n_cands < 1) return set_err(ctx, FM_ERR_INVALID, "no candidates");
    cudaSetDevice(ctx->device);
    std::vector<TileConfig> list;
    if (cands) {
        for (int i = 0; i < n_cands; ++i) {
            TileConfig t;
            const int rc = check_config(ctx, &cands[i], &t);
            if (rc) return rc;
            list.push_back(t);
        }
    } else {
        for (int lg : {2, 3, 4, 5})
            for (int cap : {12, 15, 20, 24, 32, 48, 64}) {
                TileConfig t;
                t.tw_log2 = lg;
                t.claim = 1;
                t.cap = cap;
                t.qlimit = b->cfg.qlimit;
                t.lanes = b->cfg.lanes;
                t.cap2 = b->cfg.cap2;
                list.push_back(t);
            }
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        if (e0) cudaEventDestroy(e0);
        return set_err(ctx, FM_ERR_CUDA, "event creation failed");
    }
    const TileConfig keep = b->cfg;
    TileConfig win = keep;
    float win_ms = 0.0f;
    bool have = false;
    int rc = FM_OK;
    // time one candidate: median of `reps` runs after one warm-up
    auto time_one = [&](const TileConfig& t, float& ms) -> int {
        b->cfg = t;
        int r = prepare(b);
        if (r) return r;
        r = enqueue(b, ctx->stream, false);
        if (r) return r;
        std::vector<float> v;
        for (int k = 0; k < reps; ++k) {
            FM_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
            r = enqueue(b, ctx->stream, false);
            if (r) return r;
            FM_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
            FM_CUDA(ctx, cudaEventSynchronize(e1));
            float x = 0.0f;
            FM_CUDA(ctx, cudaEventElapsedTime(&x, e0, e1));
            v.push_back(x);
        }
        std::sort(v.begin(), v.end());
        ms = v[v.size() / 2];
        return FM_OK;
    };
    for (const TileConfig& t : list) {
        float ms = 0.0f;
        if ((rc = time_one(t, ms)) != FM_OK) break;
        if (!have || ms < win_ms) {
            win = t;
            win_ms = ms;
            have = true;
        }
    }
    if (!rc && !cands) {
        // then coarser claims for the winning shape
        const TileConfig base = win;
        for (int claim : {2, 4}) {
            TileConfig t = base;
            t.claim = claim;
            float ms = 0.0f;
            if ((rc = time_one(t, ms)) != FM_OK) break;
            if (ms < win_ms) {
                win = t;
                win_ms = ms;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->cfg = rc ? keep : win;
    const int rc2 = prepare(b);
    const int rc3 = rc2 ? rc2 : capture(b);
    if (rc) return rc;
    if (rc3) return rc3;
    if (best) *best = to_public(win);
    if (best_ms) *best_ms = win_ms;
    return FM_OK;
}

int fm_batch_info_get(const fm_batch* b, fm_batch_info* out) {
    if (!b || !out) return FM_ERR_INVALID;
    fm_batch_info i{};
    i.n_views = (int32_t)b->views.size();
    i.graph_nodes = b->nodes;
    i.pixels = b->pixels;
    i.particles = b->particles;
    i.tiles = b->tiles;
    i.config = to_public(b->cfg);
    *out = i;
    return FM_OK;
}

void fm_batch_destroy(fm_batch* b) {
    if (!b) return;
    fm_ctx* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    auto& v = ctx->batches;
    v.erase(std::remove(v.begin(), v.end(), b), v.end());
    free_batch(b);
}

int fm_march_batch(fm_ctx* ctx, const fm_view* views, int32_t n_views, void* stream) {
    fm_batch* b = nullptr;
    int rc = fm_batch_create(ctx, views, n_views, nullptr, &b);
    if (rc) return rc;
    rc = fm_batch_run(b, stream);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const cudaError_t e = cudaStreamSynchronize(st);
    fm_batch_destroy(b);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(ctx, e, "cudaStreamSynchronize");
    return FM_OK;
}

}  // extern "C"
