// cg_batch.cpp -- many volumes and views per frame behind the C ABI: the
// batch render (one persistent launch), the launch-shape autotuner and the
// frame graph (every voxelize plus the batch render as one CUDA graph).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "cg_host_util.h"

namespace {

const int kLanes[4] = {1, 4, 8, 32};
const int kUnroll[3] = {1, 2, 4};
const int kBrick[3] = {4, 8, 16};

bool config_ok(const cg_trace_config* c) {
    const bool lanes = c->lanes_per_ray == 1 || c->lanes_per_ray == 4 ||
                       c->lanes_per_ray == 8 || c->lanes_per_ray == 32;
    const bool unroll = c->step_unroll == 1 || c->step_unroll == 2 || c->step_unroll == 4;
    const bool brick = c->brick == 0 || c->brick == 4 || c->brick == 8 || c->brick == 16;
    return lanes && unroll && brick;
}

// Host-side preparation of a batch: descriptors uploaded to the context's
// buffer; returns the format and the tile total.
cg_status prepare_batch(cg_context* ctx, const cg_batch_view* views, int n,
                        const cg_render_params* params, int lanes, cudaStream_t s, int& fmt,
                        unsigned& total) {
    CG_CHECK(views && n > 0 && params, CG_ERR_INVALID_ARGUMENT, "cg_render_batch: empty batch");
    cg_status st = check_params(params);
    if (st != CG_OK) return st;
    CG_CHECK(!params->use_mlp && params->pipeline == CG_PIPELINE_FUSED, CG_ERR_UNSUPPORTED,
             "cg_render_batch: renders the plain method (use_mlp = 0, fused pipeline)");
    fmt = -1;
    std::vector<BatchView>& hv = ctx->batch_host;
    hv.resize((size_t)n);
    unsigned tiles = 0;
    const cg_volume* noise_vol = nullptr;
    for (int i = 0; i < n; ++i) {
        const cg_volume* v = views[i].volume;
        CG_CHECK(v && views[i].rgba_out, CG_ERR_INVALID_ARGUMENT,
                 "cg_render_batch: view %d has no volume or output", i);
        CG_CHECK(v->ctx == ctx, CG_ERR_INVALID_ARGUMENT,
                 "cg_render_batch: view %d's volume belongs to another context", i);
        CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_render_batch: view %d not voxelized", i);
        if (fmt < 0) fmt = v->fmt;
        CG_CHECK(v->fmt == fmt, CG_ERR_UNSUPPORTED,
                 "cg_render_batch: all volumes of a batch share one storage format");
        BatchView& b = hv[(size_t)i];
        memset(&b, 0, sizeof(b));
        st = camera_of(&views[i].camera, b.cam);
        if (st != CG_OK) return st;
        b.vd = desc_of(v);
        b.tp = trace_params_of(params, v->sun_dir);
        // noise lattice tables for the first volume's box; volumes in other
        // boxes hash the lattice on the fly (same values)
        if (!noise_vol) {
            st = ensure_noise(ctx, v, b.tp, s);
            if (st != CG_OK) return st;
            noise_vol = v;
        } else {
            bool same = true;
            for (int a = 0; a < 3; ++a)
                same = same && v->wmin[a] == noise_vol->wmin[a] && v->wmax[a] == noise_vol->wmax[a];
            b.tp.nt = same ? hv[0].tp.nt : NoiseTab{};
        }
        b.cs = make_cone_schedule(b.vd, b.tp);
        b.out = reinterpret_cast<float4*>(views[i].rgba_out);
        batch_tiles(lanes, b.cam.W, b.cam.H, b.tiles_x, b.tiles_y);
        b.tile0 = tiles;
        const unsigned long long nt = (unsigned long long)b.tiles_x * (unsigned long long)b.tiles_y;
        CG_CHECK((unsigned long long)tiles + nt < 0xFFFFFFFFull, CG_ERR_OUT_OF_RANGE,
                 "cg_render_batch: too many tiles");
        tiles += (unsigned)nt;
    }
    const size_t bytes = sizeof(BatchView) * (size_t)n;
    if (ctx->batch_dev.bytes < bytes + 16) {
        CG_CUDA(cudaDeviceSynchronize());
        CG_CUDA(ctx->batch_dev.ensure(bytes + 16));
    }
    CG_CUDA(ctx->batch_pinned.ensure(bytes));
    // the previous upload from the pinned staging buffer must have finished
    CG_CUDA(cudaStreamSynchronize(s));
    memcpy(ctx->batch_pinned.p, hv.data(), bytes);
    CG_CUDA(cudaMemcpyAsync(ctx->batch_dev.p, ctx->batch_pinned.p, bytes, cudaMemcpyHostToDevice,
                            s));
    total = tiles;
    return CG_OK;
}

BatchView* batch_views_dev(cg_context* ctx) { return ctx->batch_dev.as<BatchView>(); }
unsigned* batch_counter_dev(cg_context* ctx, int n) {
    return reinterpret_cast<unsigned*>(ctx->batch_dev.as<uint8_t>() + sizeof(BatchView) * (size_t)n);
}

cg_status apply_brick(const cg_batch_view* views, int n, int brick) {
    if (brick == 0) return CG_OK;
    for (int i = 0; i < n; ++i) {
        cg_status st = cg_volume_set_occupancy_brick(const_cast<cg_volume*>(views[i].volume), brick);
        if (st != CG_OK) return st;
    }
    return CG_OK;
}

}  // namespace

extern "C" cg_status cg_context_set_trace_config(cg_context* ctx, const cg_trace_config* config) {
    CG_CHECK(ctx && config, CG_ERR_INVALID_ARGUMENT, "cg_context_set_trace_config: null pointer");
    CG_CHECK(config_ok(config), CG_ERR_OUT_OF_RANGE,
             "cg_context_set_trace_config: lanes %d / unroll %d / brick %d not supported",
             config->lanes_per_ray, config->step_unroll, config->brick);
    ctx->trace_cfg = *config;
    return CG_OK;
}

extern "C" cg_status cg_context_get_trace_config(const cg_context* ctx, cg_trace_config* config) {
    CG_CHECK(ctx && config, CG_ERR_INVALID_ARGUMENT, "cg_context_get_trace_config: null pointer");
    *config = ctx->trace_cfg;
    return CG_OK;
}

extern "C" cg_status cg_render_batch(cg_context* ctx, const cg_batch_view* views, int n,
                                     const cg_render_params* params,
                                     const cg_trace_config* config, void* stream) {
    NvtxRange nvtx_("cg_render_batch");
    CG_CHECK(ctx, CG_ERR_INVALID_ARGUMENT, "cg_render_batch: context is NULL");
    const cg_trace_config cfg = config ? *config : ctx->trace_cfg;
    CG_CHECK(config_ok(&cfg), CG_ERR_OUT_OF_RANGE,
             "cg_render_batch: lanes %d / unroll %d / brick %d not supported", cfg.lanes_per_ray,
             cfg.step_unroll, cfg.brick);
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    cg_status st = apply_brick(views, n, cfg.brick);
    if (st != CG_OK) return st;
    int fmt = 0;
    unsigned total = 0;
    st = prepare_batch(ctx, views, n, params, cfg.lanes_per_ray, s, fmt, total);
    if (st != CG_OK) return st;
    CG_LAUNCH(ctx, launch_trace_batch(fmt, cfg.lanes_per_ray, cfg.step_unroll,
                                      batch_views_dev(ctx), n, total, batch_counter_dev(ctx, n), s));
    return CG_OK;
}

extern "C" cg_status cg_autotune(cg_context* ctx, const cg_batch_view* views, int n,
                                 const cg_render_params* params, int repeats,
                                 cg_trace_config* best, float* ms) {
    NvtxRange nvtx_("cg_autotune");
    CG_CHECK(ctx && best, CG_ERR_INVALID_ARGUMENT, "cg_autotune: null pointer");
    CG_CHECK(repeats >= 1 && repeats <= 1000, CG_ERR_OUT_OF_RANGE,
             "cg_autotune: repeats %d not in [1, 1000]", repeats);
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    cudaEvent_t e0, e1;
    CG_CUDA(cudaEventCreate(&e0));
    CG_CUDA(cudaEventCreate(&e1));
    float best_ms = 0.f;
    cg_trace_config best_cfg{1, 1, 8};
    bool have = false;
    cg_status st = CG_OK;
    int k = 0;
    for (int li = 0; li < 4 && st == CG_OK; ++li)
        for (int ui = 0; ui < 3 && st == CG_OK; ++ui)
            for (int bi = 0; bi < 3 && st == CG_OK; ++bi, ++k) {
                const cg_trace_config c{kLanes[li], kUnroll[ui], kBrick[bi]};
                st = apply_brick(views, n, c.brick);
                int fmt = 0;
                unsigned total = 0;
                if (st == CG_OK)
                    st = prepare_batch(ctx, views, n, params, c.lanes_per_ray, s, fmt, total);
                if (st != CG_OK) break;
                BatchView* vd = batch_views_dev(ctx);
                unsigned* counter = batch_counter_dev(ctx, n);
                cudaError_t e = launch_trace_batch(fmt, c.lanes_per_ray, c.step_unroll, vd, n,
                                                   total, counter, s);  // warm-up
                if (e == cudaSuccess) e = cudaEventRecord(e0, s);
                for (int r = 0; r < repeats && e == cudaSuccess; ++r)
                    e = launch_trace_batch(fmt, c.lanes_per_ray, c.step_unroll, vd, n, total,
                                           counter, s);
                if (e != cudaSuccess) {
                    st = fail(CG_ERR_CUDA, "cg_autotune: %s", cudaGetErrorString(e));
                    break;
                }
                ctx->launches += (uint64_t)repeats + 1;
                float t = 0.f;
                if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                    cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) {
                    st = fail(CG_ERR_CUDA, "cg_autotune: event timing failed");
                    break;
                }
                t /= (float)repeats;
                if (ms) ms[k] = t;
                if (!have || t < best_ms) {
                    best_ms = t;
                    best_cfg = c;
                    have = true;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != CG_OK) return st;
    ctx->trace_cfg = best_cfg;
    *best = best_cfg;
    return apply_brick(views, n, best_cfg.brick);
}

// ---------------------------------------------------------------------------
// frame graph
// ---------------------------------------------------------------------------
struct cg_frame_graph {
    cg_context* ctx = nullptr;
    std::vector<cg_volume*> volumes;
    std::vector<cg_batch_view> views;
    cg_sun sun{};
    cg_render_params params{};
    cg_trace_config cfg{};
    int fmt = 0;
    unsigned total = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    DevBuf desc;                        // the graph's own batch descriptors + tile counter
    std::vector<const void*> captured;  // device buffers the graph refers to, per volume
    std::vector<bool> tex_captured;     // the captured voxelize also writes texture copies
};

namespace {

void buffers_of(const cg_volume* v, std::vector<const void*>& out) {
    const void* p[] = {v->cwr, v->q, v->thr, v->dqb, v->culled, v->blist.p,
                       v->pyr.p, v->keys.p, v->posmap.p, v->mask.p, v->occ.p, v->bdirty.p};
    out.insert(out.end(), p, p + sizeof(p) / sizeof(p[0]));
    out.push_back(reinterpret_cast<const void*>((uintptr_t)v->n));
}

void release_graph(cg_frame_graph* g) {
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    g->exec = nullptr;
    g->graph = nullptr;
}

void free_graph(cg_frame_graph* g) {
    release_graph(g);
    g->desc.release();
    delete g;
}

// One eager frame (allocations, noise tables, descriptors), then the capture.
cg_status capture(cg_frame_graph* g) {
    cg_context* ctx = g->ctx;
    cudaStream_t s = ctx->stream;
    release_graph(g);
    const bool timing = ctx->timing;
    ctx->timing = false;
    cg_status st = CG_OK;
    for (cg_volume* v : g->volumes)
        if (st == CG_OK) st = cg_voxelize(v, &g->sun, s);
    if (st == CG_OK) st = cg_render_batch(ctx, g->views.data(), (int)g->views.size(), &g->params,
                                          &g->cfg, s);
    if (st == CG_OK && cudaStreamSynchronize(s) != cudaSuccess)
        st = fail(CG_ERR_CUDA, "cg_frame_graph: eager frame failed");
    if (st != CG_OK) {
        ctx->timing = timing;
        return st;
    }
    // the graph keeps its own copy of the batch descriptors (other batch
    // renders on the context rewrite the context's)
    const int nv = (int)g->views.size();
    const size_t bytes = sizeof(BatchView) * (size_t)nv;
    if (g->desc.ensure(bytes + 16) != cudaSuccess ||
        cudaMemcpy(g->desc.p, ctx->batch_dev.p, bytes, cudaMemcpyDeviceToDevice) != cudaSuccess) {
        ctx->timing = timing;
        return fail(CG_ERR_OUT_OF_MEMORY, "cg_frame_graph: descriptor buffer");
    }
    BatchView* views_dev = g->desc.as<BatchView>();
    unsigned* counter = reinterpret_cast<unsigned*>(g->desc.as<uint8_t>() + bytes);
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (cg_volume* v : g->volumes)
            if (st == CG_OK) st = cg_voxelize(v, &g->sun, s);
        if (st == CG_OK)
            e = launch_trace_batch(g->fmt, g->cfg.lanes_per_ray, g->cfg.step_unroll, views_dev, nv,
                                   g->total, counter, s);
        cudaGraph_t graph = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(s, &graph);
        if (e == cudaSuccess) e = e2;
        g->graph = graph;
    }
    ctx->timing = timing;
    if (st != CG_OK) return st;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    CG_CHECK(e == cudaSuccess, CG_ERR_CUDA, "cg_frame_graph: capture failed: %s",
             cudaGetErrorString(e));
    g->captured.clear();
    g->tex_captured.clear();
    for (cg_volume* v : g->volumes) {
        buffers_of(v, g->captured);
        g->tex_captured.push_back(v->tex_arr[0] != nullptr);
    }
    return CG_OK;
}

}  // namespace

extern "C" cg_status cg_frame_graph_create(cg_context* ctx, cg_volume* const* volumes, int nvol,
                                           const cg_sun* sun, const cg_batch_view* views,
                                           int nviews, const cg_render_params* params,
                                           cg_frame_graph** out) {
    CG_CHECK(ctx && volumes && nvol > 0 && sun && views && nviews > 0 && params && out,
             CG_ERR_INVALID_ARGUMENT, "cg_frame_graph_create: null pointer or empty frame");
    *out = nullptr;
    CG_CUDA(cudaSetDevice(ctx->device));
    cg_frame_graph* g = new cg_frame_graph();
    g->ctx = ctx;
    g->volumes.assign(volumes, volumes + nvol);
    g->views.assign(views, views + nviews);
    g->sun = *sun;
    g->params = *params;
    g->cfg = ctx->trace_cfg;
    for (cg_volume* v : g->volumes)
        if (!v || v->ctx != ctx) {
            delete g;
            return fail(CG_ERR_INVALID_ARGUMENT, "cg_frame_graph_create: volume of another context");
        }
    for (const cg_batch_view& bv : g->views) {
        bool listed = false;
        for (cg_volume* v : g->volumes) listed = listed || bv.volume == v;
        if (!listed) {
            delete g;
            return fail(CG_ERR_INVALID_ARGUMENT,
                        "cg_frame_graph_create: a view's volume is not among the frame's volumes");
        }
    }
    // format and tile count of the batch (prepared again by the eager frame)
    cg_status st = apply_brick(g->views.data(), nviews, g->cfg.brick);
    if (st == CG_OK) {
        for (cg_volume* v : g->volumes)
            if (st == CG_OK && !v->voxelized) st = cg_voxelize(v, sun, ctx->stream);
    }
    if (st == CG_OK)
        st = prepare_batch(ctx, g->views.data(), nviews, params, g->cfg.lanes_per_ray,
                           ctx->stream, g->fmt, g->total);
    if (st == CG_OK) st = capture(g);
    if (st != CG_OK) {
        free_graph(g);
        return st;
    }
    context_retain(ctx);
    *out = g;
    return CG_OK;
}

extern "C" cg_status cg_frame_graph_launch(cg_frame_graph* g, void* stream) {
    NvtxRange nvtx_("cg_frame_graph_launch");
    CG_CHECK(g && g->exec, CG_ERR_INVALID_ARGUMENT, "cg_frame_graph_launch: no graph");
    CG_CUDA(cudaSetDevice(g->ctx->device));
    // a billboard upload that reallocated a volume's buffers invalidates the
    // captured pointers: capture again
    std::vector<const void*> now;
    for (cg_volume* v : g->volumes) buffers_of(v, now);
    if (now != g->captured) {
        cg_status st = capture(g);
        if (st != CG_OK) return st;
    }
    cudaStream_t s = pick_stream(g->ctx, stream);
    // the replay reads each volume's boards: order it after their uploads, and
    // later uploads after it
    for (cg_volume* v : g->volumes)
        if (v->ready_pending && s != g->ctx->stream)
            CG_CUDA(cudaStreamWaitEvent(s, v->boards_ready, 0));
    CG_CUDA(cudaGraphLaunch(g->exec, s));
    for (cg_volume* v : g->volumes) {
        CG_CUDA(cudaEventRecord(v->boards_read, s));
        v->read_pending = true;
    }
    g->ctx->launches += 1;
    // the replay voxelized every volume with its current billboards
    for (size_t i = 0; i < g->volumes.size(); ++i) {
        cg_volume* v = g->volumes[i];
        const bool tex_current = v->tex_gen == v->gen && g->tex_captured[i];
        v->gen++;
        v->boards_dirty = false;
        if (tex_current) v->tex_gen = v->gen;
    }
    return CG_OK;
}

extern "C" void cg_frame_graph_destroy(cg_frame_graph* g) {
    if (!g) return;
    cudaSetDevice(g->ctx->device);
    cudaDeviceSynchronize();
    cg_context* ctx = g->ctx;
    free_graph(g);
    context_release(ctx);
}
