// cg_host.cpp -- the C ABI (include/cloudgb.h): contexts, volumes, board
// quantization, pass orchestration and readback.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cg_host_util.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

cg_status fail(cg_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return s;
}

// ---------------------------------------------------------------------------
// library
// ---------------------------------------------------------------------------
extern "C" const char* cg_status_string(cg_status s) {
    switch (s) {
        case CG_OK: return "ok";
        case CG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case CG_ERR_OUT_OF_RANGE: return "out of range";
        case CG_ERR_OUT_OF_MEMORY: return "out of memory";
        case CG_ERR_CUDA: return "CUDA error";
        case CG_ERR_NOT_READY: return "not ready";
        case CG_ERR_DEVICE_FAULT: return "device fault";
        case CG_ERR_IO: return "I/O error";
        case CG_ERR_BAD_CHECKPOINT: return "bad checkpoint";
        case CG_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

extern "C" const char* cg_last_error(void) { return g_last_error.c_str(); }

void set_last_error(const char* msg) { g_last_error = msg; }
extern "C" int cg_abi_version(void) { return CLOUDGB_ABI_VERSION; }

extern "C" cg_status cg_context_create(int device, cg_context** out) {
    CG_CHECK(out, CG_ERR_INVALID_ARGUMENT, "cg_context_create: out is NULL");
    *out = nullptr;
    int ndev = 0;
    CG_CUDA(cudaGetDeviceCount(&ndev));
    CG_CHECK(device >= 0 && device < ndev, CG_ERR_OUT_OF_RANGE,
             "cg_context_create: device %d not in [0, %d)", device, ndev);
    CG_CUDA(cudaSetDevice(device));
    cg_context* c = new cg_context();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->clear_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (c->join_ev) cudaEventDestroy(c->join_ev);
        if (c->clear_ev) cudaEventDestroy(c->clear_ev);
        if (c->fork_ev) cudaEventDestroy(c->fork_ev);
        if (c->side) cudaStreamDestroy(c->side);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return fail(CG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    *out = c;
    return CG_OK;
}

void stage_begin(cg_context* ctx, cudaStream_t s) {
    if (!ctx->timing) return;
    ctx->n_marks = 0;
    stage_mark(ctx, s, "begin");
}

void stage_mark(cg_context* ctx, cudaStream_t s, const char* name) {
    if (!ctx->timing || ctx->n_marks >= 32) return;
    const int i = ctx->n_marks;
    if (!ctx->marks[i] && cudaEventCreate(&ctx->marks[i]) != cudaSuccess) return;
    if (cudaEventRecord(ctx->marks[i], s) != cudaSuccess) return;
    snprintf(ctx->mark_names[i], sizeof(ctx->mark_names[i]), "%s", name);
    ctx->n_marks = i + 1;
}

// ---- bounds-check build -------------------------------------------------
// Each kernel translation unit keeps its own error word (cg_check.cuh).
#define CG_TU_LIST(X)                                                                     \
    X(k_trace) X(k_deferred) X(k_shade_tc) X(k_render_tc) X(k_voxelize) X(k_batch)        \
    X(k_compat) X(k_mlp) X(k_textures) X(k_train_tc) X(k_noalloc) X(k_stats)
#define CG_TU_DECL(name) cudaError_t cg_oob_take_##name(unsigned long long out[2]);
CG_TU_LIST(CG_TU_DECL)

unsigned long long cg_bounds_take(char* site, int site_len, cudaError_t* err) {
    unsigned long long total = 0;
    *err = cudaSuccess;
    if (site && site_len > 0) site[0] = 0;
#define CG_TU_TAKE(name)                                                               \
    {                                                                                  \
        unsigned long long w[2] = {0ull, 0ull};                                        \
        const cudaError_t e = cg_oob_take_##name(w);                                   \
        if (e != cudaSuccess && *err == cudaSuccess) *err = e;                         \
        if (w[0] && !total && site && site_len > 0)                                    \
            snprintf(site, (size_t)site_len, "%s.cu (or a header it includes):%u index %u", \
                     #name, (unsigned)(w[1] >> 32), (unsigned)(w[1] & 0xFFFFFFFFu));    \
        total += w[0];                                                                 \
    }
    CG_TU_LIST(CG_TU_TAKE)
#undef CG_TU_TAKE
    return total;
}

extern "C" int cg_bounds_check_build(void) { return CG_BOUNDS_CHECK; }

extern "C" cg_status cg_context_bounds_violations(cg_context* ctx, uint64_t* count, char* site,
                                                  int site_len) {
    CG_CHECK(ctx && count, CG_ERR_INVALID_ARGUMENT,
             "cg_context_bounds_violations: null pointer");
    *count = 0;
    CG_CHECK(CG_BOUNDS_CHECK, CG_ERR_UNSUPPORTED,
             "cg_context_bounds_violations: not a bounds-check build");
    CG_CUDA(cudaSetDevice(ctx->device));
    CG_CUDA(cudaDeviceSynchronize());
    cudaError_t e = cudaSuccess;
    *count = cg_bounds_take(site, site_len, &e);
    CG_CUDA(e);
    return CG_OK;
}

extern "C" cg_status cg_context_last_samples(cg_context* ctx, uint64_t* samples) {
    CG_CHECK(ctx && samples, CG_ERR_INVALID_ARGUMENT, "cg_context_last_samples: null pointer");
    *samples = 0;
    if (!ctx->fallbacks.p || !ctx->shaded_valid) return CG_OK;
    CG_CUDA(cudaSetDevice(ctx->device));
    CG_CUDA(cudaDeviceSynchronize());
    unsigned long long h[3] = {0, 0, 0};
    CG_CUDA(cudaMemcpy(h, ctx->fallbacks.p, sizeof(h), cudaMemcpyDeviceToHost));
    *samples = h[2];
    return CG_OK;
}

extern "C" cg_status cg_context_set_timing(cg_context* ctx, int enable) {
    CG_CHECK(ctx, CG_ERR_INVALID_ARGUMENT, "cg_context_set_timing: ctx is NULL");
    ctx->timing = enable != 0;
    ctx->n_marks = 0;
    return CG_OK;
}

extern "C" cg_status cg_context_stage_times(cg_context* ctx, float* ms, int max_stages,
                                            int* count, char* names, size_t names_len) {
    CG_CHECK(ctx && ms && count, CG_ERR_INVALID_ARGUMENT, "cg_context_stage_times: null pointer");
    CG_CUDA(cudaSetDevice(ctx->device));
    *count = 0;
    if (names && names_len) names[0] = '\0';
    size_t used = 0;
    for (int i = 1; i < ctx->n_marks && *count < max_stages; ++i) {
        CG_CUDA(cudaEventSynchronize(ctx->marks[i]));
        float t = 0.f;
        CG_CUDA(cudaEventElapsedTime(&t, ctx->marks[i - 1], ctx->marks[i]));
        ms[(*count)++] = t;
        if (names && used + 1 < names_len) {
            int w = snprintf(names + used, names_len - used, "%s%s", i > 1 ? ";" : "",
                             ctx->mark_names[i]);
            if (w > 0) used += (size_t)w;
        }
    }
    return CG_OK;
}

void release_noise_textures(cg_context* ctx) {
    for (int o = 0; o < CG_MAX_LEVELS; ++o) {
        if (ctx->noise_tex[o]) cudaDestroyTextureObject(ctx->noise_tex[o]);
        if (ctx->noise_arr[o]) cudaFreeArray(ctx->noise_arr[o]);
        ctx->noise_tex[o] = 0;
        ctx->noise_arr[o] = nullptr;
    }
    if (ctx->fbm_tex) cudaDestroyTextureObject(ctx->fbm_tex);
    if (ctx->fbm_surf) cudaDestroySurfaceObject(ctx->fbm_surf);
    if (ctx->fbm_arr) cudaFreeArray(ctx->fbm_arr);
    ctx->fbm_tex = 0;
    ctx->fbm_surf = 0;
    ctx->fbm_arr = nullptr;
    ctx->fbm_res = 0;
    ctx->fbm_valid = false;
}

// The fBm of the current noise tables sampled at R^3 texel centres over the
// tables' noise domain (R = 8 texels per finest lattice cell, at most 512 for
// a static domain, 640 for one widened for a moving shift), as a half-precision
// 3D texture: one fetch per view sample in the surrogate path.
cg_status ensure_fbm_volume(cg_context* ctx, const cg_volume* v, TraceParams& tp, cudaStream_t s) {
    (void)v;
    if (tp.noise_octaves <= 0 || !ctx->noise_valid) return CG_OK;
    if (!ctx->fbm_valid) {
        double fmax = (double)tp.noise_freq;
        for (int o = 1; o < tp.noise_octaves; ++o) fmax *= (double)tp.noise_lac;
        float org[3], ext[3];
        double rmax = 0.0;
        for (int a = 0; a < 3; ++a) {
            org[a] = ctx->noise_dom[a];
            ext[a] = ctx->noise_dom[3 + a] - ctx->noise_dom[a];
            rmax = std::max(rmax, (double)ext[a]);
        }
        double cells = std::ceil(std::fabs(fmax) * rmax);
        const double cap = ctx->noise_moving ? 640.0 : 512.0;
        int R = (int)std::min(cap, std::max(8.0, 8.0 * cells));
        cudaChannelFormatDesc fd = cudaCreateChannelDescHalf();
        CG_CUDA(cudaMalloc3DArray(&ctx->fbm_arr, &fd, make_cudaExtent(R, R, R),
                                  cudaArraySurfaceLoadStore));
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = ctx->fbm_arr;
        CG_CUDA(cudaCreateSurfaceObject(&ctx->fbm_surf, &rd));
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModeLinear;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        CG_CUDA(cudaCreateTextureObject(&ctx->fbm_tex, &rd, &td, nullptr));
        CG_LAUNCH(ctx, launch_fbm_volume(tp, org, ext, R, ctx->fbm_surf, s));
        ctx->fbm_res = R;
        ctx->fbm_valid = true;
        ctx->noise_tab.fbm_tex = ctx->fbm_tex;
        ctx->noise_tab.fbm_res = R;
        for (int a = 0; a < 3; ++a) {
            ctx->noise_tab.fbm_org[a] = org[a];
            ctx->noise_tab.fbm_sc[a] = (float)((double)R / (double)ext[a]);
        }
    }
    tp.nt.fbm_tex = ctx->fbm_tex;
    tp.nt.fbm_res = ctx->fbm_res;
    for (int a = 0; a < 3; ++a) {
        tp.nt.fbm_org[a] = ctx->noise_tab.fbm_org[a];
        tp.nt.fbm_sc[a] = ctx->noise_tab.fbm_sc[a];
    }
    return CG_OK;
}

// Half2 (density, light) texture copies of every level for the surrogate
// renderer: arrays created on first use, refreshed after each voxelize.
cg_status ensure_textures(cg_volume* v, cudaStream_t s) {
    if (!v->tex_arr[0]) {
        for (int l = 0; l < v->L; ++l) {
            cudaChannelFormatDesc fd = cudaCreateChannelDescHalf2();
            cudaExtent ext = make_cudaExtent(v->dims[l], v->dims[l], v->dims[l]);
            CG_CUDA(cudaMalloc3DArray(&v->tex_arr[l], &fd, ext, cudaArraySurfaceLoadStore));
            cudaResourceDesc rd = {};
            rd.resType = cudaResourceTypeArray;
            rd.res.array.array = v->tex_arr[l];
            CG_CUDA(cudaCreateSurfaceObject(&v->tex_surf[l], &rd));
            cudaTextureDesc td = {};
            td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;
            td.filterMode = cudaFilterModeLinear;
            td.readMode = cudaReadModeElementType;
            td.normalizedCoords = 0;
            CG_CUDA(cudaCreateTextureObject(&v->tex_obj[l], &rd, &td, nullptr));
        }
    }
    if (v->tex_gen != v->gen) {
        const VolDesc vd = desc_of(v);
        for (int l = 0; l < v->L; ++l)
            CG_LAUNCH(v->ctx, launch_pack_level(vd, l, v->tex_surf[l], s));
        v->tex_gen = v->gen;
    }
    return CG_OK;
}

// Volumes and models hold a reference on their context, so the context's
// resources outlive every object created on it whatever the destroy order.
void context_retain(cg_context* ctx) { ctx->refs++; }

void context_release(cg_context* ctx) {
    if (--ctx->refs > 0) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaStreamSynchronize(ctx->side);
    ctx->image.release();
    ctx->noise.release();
    ctx->samples_pw.release();
    ctx->samples_gl.release();
    ctx->samples_c.release();
    ctx->samples_cnt.release();
    ctx->samples_alpha.release();
    ctx->fallbacks.release();
    ctx->stats_scratch.release();
    ctx->stats_a.release();
    ctx->stats_ref.release();
    ctx->batch_pinned.release();
    ctx->batch_dev.release();
    ctx->compat_noise.release();
    ctx->compat_rect.release();
    ctx->compat_key.release();
    ctx->compat_tiles.release();
    ctx->compat_list.release();
    ctx->compat_total.release();
    release_noise_textures(ctx);
    for (cudaEvent_t e : ctx->marks)
        if (e) cudaEventDestroy(e);
    cudaEventDestroy(ctx->fork_ev);
    cudaEventDestroy(ctx->join_ev);
    cudaEventDestroy(ctx->clear_ev);
    cudaStreamDestroy(ctx->side);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" void cg_context_destroy(cg_context* ctx) {
    if (!ctx) return;
    context_release(ctx);
}

cudaStream_t pick_stream(cg_context* ctx, void* stream) {
    return stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->stream;
}

extern "C" cg_status cg_context_synchronize(cg_context* ctx) {
    CG_CHECK(ctx, CG_ERR_INVALID_ARGUMENT, "cg_context_synchronize: ctx is NULL");
    CG_CUDA(cudaSetDevice(ctx->device));
    CG_CUDA(cudaDeviceSynchronize());
    return CG_OK;
}

extern "C" uint64_t cg_context_launch_count(const cg_context* ctx) {
    return ctx ? ctx->launches : 0;
}

extern "C" void cg_render_params_default(cg_render_params* p) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->view_steps = 64;
    p->sun_steps = 24;
    p->cone_half_angle = 0.03f;
    p->cone_initial_height = 1.0f;
    p->cone_min_radius = 2.0f;
    p->lod_offset = 0.0f;
    p->down_scaling = 1.0f;
    p->density_scale = 4.0f;
    p->ambient = 0.3f;
    p->sun_color[0] = p->sun_color[1] = p->sun_color[2] = 1.0f;
    p->transmittance_cutoff = 1e-5f;
    p->cone_mode = CG_CONE_TRANSMITTANCE;
    p->noise.seed = 1;
    p->noise.octaves = 0;
    p->noise.frequency = 4.0f;
    p->noise.lacunarity = 2.0f;
    p->noise.gain = 0.5f;
    p->noise.offset[0] = p->noise.offset[1] = p->noise.offset[2] = 0.0f;
    p->use_mlp = 0;
    p->mlp = nullptr;
    p->pipeline = CG_PIPELINE_FUSED;
    // warp-cooperative cones at steps where at most 8 rays of a warp
    // contribute: the fastest threshold measured at 1080p over 256^3
    p->cone_lanes = 8;
}

extern "C" cg_status cg_host_alloc(size_t bytes, void** out) {
    CG_CHECK(out, CG_ERR_INVALID_ARGUMENT, "cg_host_alloc: out is NULL");
    CG_CUDA(cudaMallocHost(out, bytes ? bytes : 16));
    return CG_OK;
}
extern "C" void cg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}
extern "C" cg_status cg_device_alloc(size_t bytes, void** out) {
    CG_CHECK(out, CG_ERR_INVALID_ARGUMENT, "cg_device_alloc: out is NULL");
    CG_CUDA(cudaMalloc(out, bytes ? bytes : 16));
    return CG_OK;
}
extern "C" void cg_device_free(void* p) {
    if (p) cudaFree(p);
}
extern "C" cg_status cg_memcpy(void* dst, const void* src, size_t bytes, int kind) {
    CG_CHECK(dst && src, CG_ERR_INVALID_ARGUMENT, "cg_memcpy: null pointer");
    CG_CUDA(cudaMemcpy(dst, src, bytes, (cudaMemcpyKind)kind));
    return CG_OK;
}

// ---------------------------------------------------------------------------
// CloudVolume
// ---------------------------------------------------------------------------
extern "C" cg_status cg_volume_create(cg_context* ctx, int dimension, float bound_min,
                                      float bound_max, const float position[3], int mips,
                                      int format, cg_volume** out) {
    CG_CHECK(ctx && position && out, CG_ERR_INVALID_ARGUMENT, "cg_volume_create: null pointer");
    *out = nullptr;
    CG_CHECK(dimension >= 2 && dimension <= 512, CG_ERR_OUT_OF_RANGE,
             "cg_volume_create: dimension %d not in [2, 512]", dimension);
    int maxl = 1;
    while ((dimension >> maxl) >= 1 && maxl < CG_MAX_LEVELS) maxl++;
    CG_CHECK(mips >= 1 && mips <= maxl, CG_ERR_OUT_OF_RANGE,
             "cg_volume_create: mips %d not in [1, %d]", mips, maxl);
    CG_CHECK(format == CG_FORMAT_RGBA32F || format == CG_FORMAT_BF16_FP16,
             CG_ERR_INVALID_ARGUMENT, "cg_volume_create: unknown format %d", format);
    CG_CHECK(std::isfinite(bound_min) && std::isfinite(bound_max) && bound_max > bound_min,
             CG_ERR_INVALID_ARGUMENT, "cg_volume_create: bounds must be finite, min < max");
    for (int a = 0; a < 3; ++a)
        CG_CHECK(std::isfinite(position[a]), CG_ERR_INVALID_ARGUMENT,
                 "cg_volume_create: non-finite position");
    CG_CUDA(cudaSetDevice(ctx->device));
    cg_volume* v = new cg_volume();
    v->ctx = ctx;
    context_retain(ctx);
    v->D = dimension;
    v->L = mips;
    v->fmt = format;
    v->b0 = bound_min;
    v->b1 = bound_max;
    for (int a = 0; a < 3; ++a) {
        v->pos[a] = position[a];
        v->wmin[a] = position[a] + bound_min;
        v->wmax[a] = position[a] + bound_max;
        v->range[a] = v->wmax[a] - v->wmin[a];
    }
    size_t off = 0;
    for (int l = 0; l < mips; ++l) {
        int n = dimension >> l;
        if (n < 1) n = 1;
        v->dims[l] = n;
        v->offs[l] = off;
        off += (size_t)n * n * n;
    }
    for (int l = mips; l < CG_MAX_LEVELS; ++l) {
        v->dims[l] = 0;
        v->offs[l] = off;
    }
    v->total = off;
    const size_t n0 = (size_t)dimension * dimension * dimension;
    const size_t bpv = format == CG_FORMAT_RGBA32F ? 16 : 4;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = v->pyr.ensure(off * bpv);
    if (e == cudaSuccess) e = v->count.ensure(n0 * 4);
    if (e == cudaSuccess) e = v->dq.ensure(n0 * 4);
    if (e == cudaSuccess) e = v->mask.ensure(n0);
    if (e == cudaSuccess) e = v->scratch.ensure(64);
    // raw 4^3-cell grids (written by the splat) followed by the dilated brick
    // grids (at most as many bytes as the raw ones: bricks are >= 4 texels)
    int raw_total = 0;
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        int nbl = l < mips ? (v->dims[l] + 3) / 4 : 0;
        v->raw_nb[l] = nbl;
        v->raw_off[l] = raw_total;
        raw_total += nbl * nbl * nbl;
    }
    v->raw_total = raw_total;
    set_occ_layout(v, 4);  // the autotuner's pick on the batching and 1080p workloads
    // + the level-0 occupied box (6 ints) after the grids, 16-byte aligned
    if (e == cudaSuccess) e = v->occ.ensure(occ_box_offset(raw_total) + 32);
    const int nb = (dimension + CG_BRICK - 1) / CG_BRICK;
    v->bins.nbx = v->bins.nby = v->bins.nbz = nb;
    v->bins.nbricks = nb * nb * nb;
    if (e == cudaSuccess) e = v->bcount.ensure((size_t)v->bins.nbricks * 4);
    if (e == cudaSuccess) e = v->boff.ensure(((size_t)v->bins.nbricks + 1) * 4);
    if (e == cudaSuccess) e = v->bcursor.ensure((size_t)v->bins.nbricks * 4);
    // every brick starts dirty: the pyramid's memory is uninitialised
    if (e == cudaSuccess) e = v->bdirty.ensure((size_t)v->bins.nbricks);
    if (e == cudaSuccess) e = cudaMemset(v->bdirty.p, 1, (size_t)v->bins.nbricks);
    if (e == cudaSuccess) e = v->bhl.ensure((size_t)v->bins.nbricks);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->boards_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->boards_read, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cg_volume_destroy(v);
        return fail(e == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA,
                    "cg_volume_create: %s", cudaGetErrorString(e));
    }
    *out = v;
    return CG_OK;
}

extern "C" void cg_volume_destroy(cg_volume* v) {
    if (!v) return;
    cudaSetDevice(v->ctx->device);
    cudaStreamSynchronize(v->ctx->stream);
    DevBuf* bufs[] = {&v->pyr, &v->count, &v->dq, &v->mask, &v->boards,
                      &v->bcount, &v->boff, &v->bcursor, &v->blist,
                      &v->bdirty, &v->bhl,
                      &v->keys, &v->posmap, &v->scratch, &v->occ};
    for (DevBuf* b : bufs) b->release();
    v->h_stage.release();
    if (v->boards_ready) cudaEventDestroy(v->boards_ready);
    if (v->boards_read) cudaEventDestroy(v->boards_read);
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        if (v->tex_obj[l]) cudaDestroyTextureObject(v->tex_obj[l]);
        if (v->tex_surf[l]) cudaDestroySurfaceObject(v->tex_surf[l]);
        if (v->tex_arr[l]) cudaFreeArray(v->tex_arr[l]);
    }
    cg_context* ctx = v->ctx;
    delete v;
    context_release(ctx);
}

static long long floor_div_ll(long long a, long long b) {
    long long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

static bool axis_range_host(long long q, long long rq, int D, int& lo, int& hi) {
    long long l = floor_div_ll(q - rq - CG_HALF_Q20 + CG_Q20 - 1, CG_Q20);
    long long h = floor_div_ll(q + rq - CG_HALF_Q20, CG_Q20);
    if (l < 0) l = 0;
    if (h > D - 1) h = D - 1;
    if (l > h) return false;
    lo = (int)l;
    hi = (int)h;
    return true;
}

// Board quantization to the Q20 voxel grid (FP64, round to nearest even):
//   v = (cw - wmin) / range * D per axis, q = rint(v * 2^20), culled from
//   coverage when v is outside [-D, 2D];  rq = rint(r / range_x * D * 2^20),
//   error when r > range_x;  thr = floor(rq^2 * 9999 / 10000) (the 0.01
//   profile discard of first_voxelize.glsl:46);  dq = rint(density * 2^16).
extern "C" cg_status cg_volume_set_billboards(cg_volume* v, const float* positions,
                                              const float* scales, const float* densities,
                                              int count, float fluffiness) {
    CG_CHECK(v, CG_ERR_INVALID_ARGUMENT, "cg_volume_set_billboards: volume is NULL");
    CG_CHECK(count >= 0 && count <= (1 << 24), CG_ERR_OUT_OF_RANGE,
             "cg_volume_set_billboards: count %d not in [0, 2^24]", count);
    CG_CHECK(count == 0 || (positions && scales), CG_ERR_INVALID_ARGUMENT,
             "cg_volume_set_billboards: null positions/scales");
    CG_CHECK(std::isfinite(fluffiness) && fluffiness >= 0.f, CG_ERR_INVALID_ARGUMENT,
             "cg_volume_set_billboards: fluffiness must be finite and >= 0");
    CG_CUDA(cudaSetDevice(v->ctx->device));
    // a voxelize still running on another stream reads the board buffers that
    // this upload overwrites (or reallocates): wait for it
    if (v->read_pending) {
        CG_CUDA(cudaEventSynchronize(v->boards_read));
        v->read_pending = false;
    }
    v->boards_dirty = true;  // the last voxelize's bins refer to the old list
    const size_t n = (size_t)count;
    const size_t bytes_cwr = n * 16, bytes_q = n * 16, bytes_thr = n * 8, bytes_dq = n * 4,
                 bytes_cul = n;
    const size_t o_cwr = 0, o_q = o_cwr + bytes_cwr, o_thr = o_q + bytes_q,
                 o_dq = o_thr + bytes_thr, o_cul = o_dq + bytes_dq;
    const size_t total = o_cul + bytes_cul;
    CG_CUDA(cudaStreamSynchronize(v->ctx->stream));  // staging buffer reuse
    CG_CUDA(v->h_stage.ensure(total + 16));
    char* st = reinterpret_cast<char*>(v->h_stage.p);
    float* cwr = reinterpret_cast<float*>(st + o_cwr);
    int* qv = reinterpret_cast<int*>(st + o_q);
    uint64_t* thr = reinterpret_cast<uint64_t*>(st + o_thr);
    uint32_t* dqv = reinterpret_cast<uint32_t*>(st + o_dq);
    uint8_t* cul = reinterpret_cast<uint8_t*>(st + o_cul);
    const int D = v->D;
    size_t pairs = 0;
    for (size_t b = 0; b < n; ++b) {
        float r = scales[b] * fluffiness;
        float d = densities ? densities[b] : 1.0f;
        CG_CHECK(std::isfinite(r) && r >= 0.f, CG_ERR_INVALID_ARGUMENT,
                 "billboard %zu: radius must be finite and >= 0", b);
        CG_CHECK(std::isfinite(d) && d >= 0.f && d < 32768.f, CG_ERR_INVALID_ARGUMENT,
                 "billboard %zu: density must be in [0, 32768)", b);
        bool cull = false;
        long long q[3];
        for (int a = 0; a < 3; ++a) {
            float c = v->pos[a] + positions[3 * b + a];
            CG_CHECK(std::isfinite(c), CG_ERR_INVALID_ARGUMENT,
                     "billboard %zu: non-finite position", b);
            cwr[4 * b + a] = c;
            double vv = ((double)c - (double)v->wmin[a]) / (double)v->range[a] * (double)D;
            if (!(vv >= -(double)D && vv <= 2.0 * (double)D)) {
                cull = true;
                q[a] = 0;
            } else {
                q[a] = llrint(vv * (double)CG_Q20);
            }
        }
        cwr[4 * b + 3] = r;
        double rv = (double)r / (double)v->range[0] * (double)D;
        CG_CHECK(rv <= (double)D, CG_ERR_OUT_OF_RANGE,
                 "billboard %zu: radius %g exceeds the volume extent", b, (double)r);
        long long rq = llrint(rv * (double)CG_Q20);
        // rq <= 512 * 2^20 < 2^30, so rq^2 < 2^60 fits; floor(r2 * 9999 / 10000)
        // = r2 - ceil(r2 / 10000) without a 128-bit division
        const uint64_t r2 = (uint64_t)rq * (uint64_t)rq;
        thr[b] = r2 - (r2 + 9999u) / 10000u;
        dqv[b] = (uint32_t)llrint((double)d * 65536.0);
        for (int a = 0; a < 3; ++a) qv[4 * b + a] = (int)q[a];
        qv[4 * b + 3] = (int)rq;
        int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        if (!cull)
            for (int a = 0; a < 3; ++a)
                if (!axis_range_host(q[a], rq, D, lo[a], hi[a])) cull = true;
        cul[b] = cull ? 1 : 0;
        if (!cull) {
            size_t nbz = (size_t)(hi[2] / CG_BRICK - lo[2] / CG_BRICK + 1);
            size_t nby = (size_t)(hi[1] / CG_BRICK - lo[1] / CG_BRICK + 1);
            size_t nbx = (size_t)(hi[0] / CG_BRICK - lo[0] / CG_BRICK + 1);
            pairs += nbx * nby * nbz;
        }
    }
    CG_CHECK(pairs < (size_t)0xFFFFFFFFu, CG_ERR_OUT_OF_RANGE,
             "cg_volume_set_billboards: %zu board-brick pairs exceed 2^32", pairs);
    // the device records mirror the staging layout: one copy uploads them all
    CG_CUDA(v->boards.ensure(total));
    char* dev = v->boards.as<char>();
    v->cwr = reinterpret_cast<float4*>(dev + o_cwr);
    v->q = reinterpret_cast<int4*>(dev + o_q);
    v->thr = reinterpret_cast<uint64_t*>(dev + o_thr);
    v->dqb = reinterpret_cast<uint32_t*>(dev + o_dq);
    v->culled = reinterpret_cast<uint8_t*>(dev + o_cul);
    CG_CUDA(v->blist.ensure(pairs * 4));
    cudaStream_t s = v->ctx->stream;
    if (n) CG_CUDA(cudaMemcpyAsync(dev, st, total, cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaEventRecord(v->boards_ready, s));
    v->ready_pending = true;
    v->n = count;
    v->pairs = pairs;
    v->voxelized = false;
    return CG_OK;
}

BoardsDev boards_of(const cg_volume* v) {
    BoardsDev b;
    b.n = v->n;
    b.cwr = v->cwr;
    b.q = v->q;
    b.thr = v->thr;
    b.dq = v->dqb;
    b.culled = v->culled;
    return b;
}

// Brick grids of edge `brick` (4, 8 or 16) per level.
void set_occ_layout(cg_volume* v, int brick) {
    v->occ_brick = brick;
    int total = 0;
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        int nbl = l < v->L ? (v->dims[l] + brick - 1) / brick : 0;
        v->occ_nb[l] = nbl;
        v->occ_off[l] = total;
        total += nbl * nbl * nbl;
    }
    v->occ_total = total;
}

OccRaw raw_of(const cg_volume* v) {
    OccRaw r;
    r.raw = v->occ.as<uint8_t>();
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        r.nb[l] = v->raw_nb[l];
        r.off[l] = v->raw_off[l];
    }
    return r;
}

size_t occ_box_offset(int raw_total) { return ((2 * (size_t)raw_total) + 15) & ~(size_t)15; }

VolDesc desc_of(const cg_volume* v) {
    VolDesc d;
    d.D = v->D;
    d.L = v->L;
    d.fmt = v->fmt;
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        d.dims[l] = v->dims[l];
        d.offs[l] = (long long)v->offs[l];
        d.lsc[l] = l < v->L ? (float)v->dims[l] / (float)v->D : 0.f;
    }
    for (int a = 0; a < 3; ++a) {
        d.wmin[a] = v->wmin[a];
        d.range[a] = v->range[a];
    }
    d.pyr = v->pyr.p;
    d.occ = v->occ.as<const uint8_t>() + v->raw_total;
    d.occ_box = reinterpret_cast<const int*>(v->occ.as<const uint8_t>() +
                                             occ_box_offset(v->raw_total));
    d.occ_shift = v->occ_brick == 4 ? 2 : (v->occ_brick == 16 ? 4 : 3);
    for (int l = 0; l < CG_MAX_LEVELS; ++l) d.tex[l] = v->tex_obj[l];
    for (int l = 0; l < CG_MAX_LEVELS; ++l) d.surf[l] = 0;
    for (int l = 0; l < CG_MAX_LEVELS; ++l) {
        d.occ_nb[l] = v->occ_nb[l];
        d.occ_off[l] = v->occ_off[l];
    }
    d.nvox = (long long)v->offs[v->L - 1] +
             (long long)v->dims[v->L - 1] * v->dims[v->L - 1] * v->dims[v->L - 1];
    d.occ_total = (int)v->occ_total;
    return d;
}

// FP32 vector helpers in GLM's operation order; this translation unit is
// compiled with -ffp-contract=off so that the frame is bit-identical to the
// oracle's.
struct V3 {
    float x, y, z;
};
static float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static V3 cross3(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
static V3 normalize3(V3 v) {
    float inv = 1.0f / std::sqrt(dot3(v, v));
    return {v.x * inv, v.y * inv, v.z * inv};
}

// Sun::update (Sun.hpp:26-43) for a directional sun: lookDir = -s, lookPos =
// position - lookDir * max(|min|, |max|), V = lookAt(lookPos, position, +y),
// ortho box [2 minComp, 2 maxComp]^2, near 0.01.
bool sun_frame_for_box(const float position[3], float b0, float b1, const float dir[3], int W,
                       int H, SunFrame& fr) {
    V3 pos{position[0], position[1], position[2]};
    V3 lookDir = normalize3({-dir[0], -dir[1], -dir[2]});
    V3 mn{b0, b0, b0}, mx{b1, b1, b1};
    float minLen = std::sqrt(dot3(mn, mn)), maxLen = std::sqrt(dot3(mx, mx));
    float dist = minLen > maxLen ? minLen : maxLen;
    V3 lookPos{pos.x - lookDir.x * dist, pos.y - lookDir.y * dist, pos.z - lookDir.z * dist};
    V3 f = normalize3({pos.x - lookPos.x, pos.y - lookPos.y, pos.z - lookPos.z});
    V3 c = cross3(f, {0.0f, 1.0f, 0.0f});
    float cl = dot3(c, c);
    if (!(cl > 1e-12f)) return false;
    V3 r = normalize3(c);
    V3 u = cross3(r, f);
    fr.eye[0] = lookPos.x; fr.eye[1] = lookPos.y; fr.eye[2] = lookPos.z;
    fr.right[0] = r.x; fr.right[1] = r.y; fr.right[2] = r.z;
    fr.up[0] = u.x; fr.up[1] = u.y; fr.up[2] = u.z;
    fr.fwd[0] = f.x; fr.fwd[1] = f.y; fr.fwd[2] = f.z;
    fr.t[0] = -dot3(r, lookPos);
    fr.t[1] = -dot3(u, lookPos);
    fr.t[2] = dot3(f, lookPos);
    fr.lo = 2.0f * b0;
    fr.hi = 2.0f * b1;
    fr.near_z = 0.01f;
    V3 np{lookPos.x + lookDir.x * 0.01f, lookPos.y + lookDir.y * 0.01f,
          lookPos.z + lookDir.z * 0.01f};
    float two_d = 2.0f * dist;
    V3 fp{lookPos.x + lookDir.x * two_d, lookPos.y + lookDir.y * two_d,
          lookPos.z + lookDir.z * two_d};
    V3 dd{np.x - fp.x, np.y - fp.y, np.z - fp.z};
    fr.clip = std::sqrt(dot3(dd, dd));
    fr.W = W;
    fr.H = H;
    return true;
}

static bool make_sun_frame(const cg_volume* v, const float dir[3], int W, int H, SunFrame& fr) {
    return sun_frame_for_box(v->pos, v->b0, v->b1, dir, W, H, fr);
}

// stepSize = min(voxelSize) (VoxelizeShader.cpp:128); offset along each axis
// of stepSize * normalize(+-1,+-1,+-1) (second_voxelize.glsl:42-49).
static float highlight_offset(const cg_volume* v) {
    float vs0 = v->range[0] / (float)v->D, vs1 = v->range[1] / (float)v->D,
          vs2 = v->range[2] / (float)v->D;
    float step = vs0 < vs1 ? vs0 : vs1;
    step = step < vs2 ? step : vs2;
    return step * 0.57735026f;
}


extern "C" cg_status cg_voxelize(cg_volume* v, const cg_sun* sun, void* stream) {
    NvtxRange nvtx_("cg_voxelize");
    CG_CHECK(v && sun, CG_ERR_INVALID_ARGUMENT, "cg_voxelize: null pointer");
    CG_CHECK(sun->map_width >= 1 && sun->map_height >= 1 && sun->map_width <= 16384 &&
                 sun->map_height <= 16384,
             CG_ERR_OUT_OF_RANGE, "cg_voxelize: sun map %dx%d not in [1, 16384]^2",
             sun->map_width, sun->map_height);
    for (int a = 0; a < 3; ++a)
        CG_CHECK(std::isfinite(sun->direction[a]), CG_ERR_INVALID_ARGUMENT,
                 "cg_voxelize: non-finite sun direction");
    SunFrame fr;
    CG_CHECK(make_sun_frame(v, sun->direction, sun->map_width, sun->map_height, fr),
             CG_ERR_INVALID_ARGUMENT,
             "cg_voxelize: sun direction is zero or parallel to the up axis (0,1,0)");
    cg_context* ctx = v->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t texels = (size_t)sun->map_width * sun->map_height;
    if (v->mapW != sun->map_width || v->mapH != sun->map_height) {
        CG_CUDA(cudaStreamSynchronize(s));
        CG_CUDA(v->keys.ensure(texels * 8));
        CG_CUDA(v->posmap.ensure(texels * 16));
        v->mapW = sun->map_width;
        v->mapH = sun->map_height;
    }
    v->frame = fr;
    for (int a = 0; a < 3; ++a) v->sun_dir[a] = sun->direction[a];
    const size_t n0 = (size_t)v->D * v->D * v->D;
    BoardsDev b = boards_of(v);
    Bins bins = v->bins;
    bins.count = v->bcount.as<uint32_t>();
    bins.offset = v->boff.as<uint32_t>();
    bins.cursor = v->bcursor.as<uint32_t>();
    bins.list = v->blist.as<uint32_t>();
    bins.dirty = v->bdirty.as<uint8_t>();
    bins.hl = v->bhl.as<const uint8_t>();
    VolDesc vd = desc_of(v);
    // once the surrogate renderer has built the texture copies, keep them
    // current from the voxelize stores instead of a copy pass
    const bool write_tex = v->tex_arr[0] != nullptr;
    if (write_tex)
        for (int l = 0; l < v->L; ++l) vd.surf[l] = v->tex_surf[l];
    // order after the last board upload (made on the context stream); a
    // stream being captured into a graph is ordered at graph launch instead
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CG_CUDA(cudaStreamIsCapturing(s, &cap));
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    if (v->ready_pending && s != ctx->stream && !capturing)
        CG_CUDA(cudaStreamWaitEvent(s, v->boards_ready, 0));
    stage_begin(ctx, s);
    // the sun-view pass does not need the bins: it runs on the side stream
    // while the binning (latency-bound, a few SMs busy) runs on s
    cudaStream_t sd = ctx->side;
    CG_CUDA(cudaEventRecord(ctx->fork_ev, s));
    CG_CUDA(cudaStreamWaitEvent(sd, ctx->fork_ev, 0));
    // clearGPU (CloudVolume.cpp:96-100) + clearPositionMap (VoxelizeShader.cpp:185-187):
    // the highlight mask and its brick flags are cleared on s, where the binning
    // has time to spare, the key map on the side stream ahead of the sun map
    CG_CUDA(cudaMemsetAsync(v->mask.p, 0, n0, s));
    CG_CUDA(cudaMemsetAsync(v->bhl.p, 0, (size_t)bins.nbricks, s));
    CG_CUDA(cudaEventRecord(ctx->clear_ev, s));
    CG_CUDA(cudaMemsetAsync(v->keys.p, 0xFF, texels * 8, sd));
    {
        NvtxRange r("voxelize.sun_pass");
        // pass 1: sun-view nearest-surface map
        if (b.n) CG_LAUNCH(ctx, launch_sunmap(b, fr, v->keys.as<uint64_t>(), sd));
        // pass 2: highlight stores (after the mask's clearing)
        CG_CUDA(cudaStreamWaitEvent(sd, ctx->clear_ev, 0));
        CG_LAUNCH(ctx, launch_highlight(b, fr, v->keys.as<uint64_t>(), v->posmap.as<float4>(),
                                        v->D, v->wmin, v->range, highlight_offset(v),
                                        v->mask.as<uint8_t>(), v->bhl.as<uint8_t>(), sd));
        CG_CUDA(cudaEventRecord(ctx->join_ev, sd));
    }
    {
        NvtxRange r("voxelize.bins");
        CG_CUDA(cudaMemsetAsync(bins.count, 0, (size_t)bins.nbricks * 4, s));
        // raw cells, brick grids (rewritten by the dilation) and the occupied box
        CG_CUDA(cudaMemsetAsync(v->occ.p, 0, occ_box_offset(v->raw_total) + 6 * sizeof(int), s));
        // brick bins
        if (b.n) CG_LAUNCH(ctx, launch_bin_count(b, v->D, bins, s));
        CG_LAUNCH(ctx, launch_bin_scan(bins, s));
        if (b.n) CG_LAUNCH(ctx, launch_bin_fill(b, v->D, bins, s));
    }
    stage_mark(ctx, s, "bins");
    CG_CUDA(cudaStreamWaitEvent(s, ctx->join_ev, 0));
    // the sun-view pass's time beyond the binning
    stage_mark(ctx, s, "sun");
    // coverage splat + level 0 + fused mips
    int fused = (v->D % CG_BRICK == 0) ? std::min(CG_FUSED_MIPS, v->L - 1) : 0;
    {
        NvtxRange r("voxelize.splat");
        CG_LAUNCH(ctx, launch_splat(b, bins, v->mask.as<uint8_t>(), vd, v->pyr.p,
                                    v->count.as<uint32_t>(), v->dq.as<uint32_t>(), fused,
                                    raw_of(v), false, s));
    }
    stage_mark(ctx, s, "splat");
    // the occupancy dilation (raw cells -> brick grids, occupied box) and the
    // remaining mips are independent: the dilation runs on the side stream
    CG_CUDA(cudaEventRecord(ctx->fork_ev, s));
    CG_CUDA(cudaStreamWaitEvent(sd, ctx->fork_ev, 0));
    CG_LAUNCH(ctx, launch_occ_dilate(vd, raw_of(v), v->occ.as<uint8_t>() + v->raw_total,
                                     v->occ_total, sd));
    CG_CUDA(cudaEventRecord(ctx->join_ev, sd));
    // remaining mips (glGenerateMipmap, VoxelizeShader.cpp:105)
    {
        int l = fused;
        for (; l + 1 < v->L; ++l) {
            const long long np = v->dims[l + 1];
            if (np * np * np <= CG_MIP_TAIL_MAX) break;
            CG_LAUNCH(ctx, launch_mip_level(vd, v->pyr.p, l, s));
        }
        if (l + 1 < v->L) CG_LAUNCH(ctx, launch_mip_tail(vd, v->pyr.p, l, s));
    }
    CG_CUDA(cudaStreamWaitEvent(s, ctx->join_ev, 0));
    stage_mark(ctx, s, "mips");
    if (!capturing) {
        CG_CUDA(cudaEventRecord(v->boards_read, s));
        v->read_pending = true;
    }
    v->voxelized = true;
    v->boards_dirty = false;
    v->gen++;
    if (write_tex) v->tex_gen = v->gen;
    return CG_OK;
}

// ---------------------------------------------------------------------------
// render
// ---------------------------------------------------------------------------
cg_status check_params(const cg_render_params* p) {
    CG_CHECK(p->view_steps >= 1 && p->view_steps <= 4096, CG_ERR_OUT_OF_RANGE,
             "render params: view_steps %d not in [1, 4096]", p->view_steps);
    CG_CHECK(p->sun_steps >= 0 && p->sun_steps <= 64, CG_ERR_OUT_OF_RANGE,
             "render params: sun_steps %d not in [0, 64]", p->sun_steps);
    CG_CHECK(std::isfinite(p->cone_half_angle) && p->cone_half_angle >= 0.f &&
                 p->cone_half_angle < 1.5f,
             CG_ERR_OUT_OF_RANGE, "render params: cone_half_angle not in [0, 1.5)");
    CG_CHECK(std::isfinite(p->cone_initial_height) && p->cone_initial_height >= 0.f,
             CG_ERR_INVALID_ARGUMENT, "render params: cone_initial_height must be >= 0");
    CG_CHECK(std::isfinite(p->cone_min_radius) && p->cone_min_radius >= 0.f,
             CG_ERR_INVALID_ARGUMENT, "render params: cone_min_radius must be >= 0");
    CG_CHECK(std::isfinite(p->lod_offset), CG_ERR_INVALID_ARGUMENT,
             "render params: lod_offset must be finite");
    CG_CHECK(std::isfinite(p->down_scaling) && p->down_scaling > 0.f, CG_ERR_INVALID_ARGUMENT,
             "render params: down_scaling must be > 0");
    CG_CHECK(std::isfinite(p->density_scale) && p->density_scale >= 0.f,
             CG_ERR_INVALID_ARGUMENT, "render params: density_scale must be >= 0");
    CG_CHECK(std::isfinite(p->ambient) && p->ambient >= 0.f && p->ambient <= 1.f,
             CG_ERR_OUT_OF_RANGE, "render params: ambient not in [0, 1]");
    CG_CHECK(std::isfinite(p->transmittance_cutoff) && p->transmittance_cutoff >= 0.f &&
                 p->transmittance_cutoff < 1.f,
             CG_ERR_OUT_OF_RANGE, "render params: transmittance_cutoff not in [0, 1)");
    CG_CHECK(p->cone_mode == CG_CONE_TRANSMITTANCE || p->cone_mode == CG_CONE_REFERENCE,
             CG_ERR_INVALID_ARGUMENT, "render params: unknown cone_mode %d", p->cone_mode);
    CG_CHECK(p->pipeline == CG_PIPELINE_FUSED || p->pipeline == CG_PIPELINE_DEFERRED ||
                 p->pipeline == CG_PIPELINE_PERSISTENT,
             CG_ERR_INVALID_ARGUMENT, "render params: unknown pipeline %d", p->pipeline);
    CG_CHECK(p->cone_lanes >= 0 && p->cone_lanes <= 32, CG_ERR_OUT_OF_RANGE,
             "render params: cone_lanes %d not in [0, 32]", p->cone_lanes);
    CG_CHECK(p->pipeline != CG_PIPELINE_PERSISTENT || p->use_mlp, CG_ERR_UNSUPPORTED,
             "render params: the persistent pipeline renders the MLP surrogate only");
    CG_CHECK(p->noise.octaves >= 0 && p->noise.octaves <= 16, CG_ERR_OUT_OF_RANGE,
             "render params: noise octaves %d not in [0, 16]", p->noise.octaves);
    CG_CHECK(std::isfinite(p->noise.frequency) && std::isfinite(p->noise.lacunarity) &&
                 std::isfinite(p->noise.gain) && p->noise.gain > 0.f,
             CG_ERR_INVALID_ARGUMENT, "render params: noise values must be finite, gain > 0");
    for (int a = 0; a < 3; ++a)
        CG_CHECK(std::isfinite(p->noise.offset[a]) && std::fabs(p->noise.offset[a]) < 1e6f,
                 CG_ERR_OUT_OF_RANGE, "render params: noise offset must be finite, |offset| < 1e6");
    for (int a = 0; a < 3; ++a)
        CG_CHECK(std::isfinite(p->sun_color[a]), CG_ERR_INVALID_ARGUMENT,
                 "render params: non-finite sun colour");
    return CG_OK;
}

TraceParams trace_params_of(const cg_render_params* p, const float sun_dir[3]) {
    TraceParams tp;
    tp.view_steps = p->view_steps;
    tp.sun_steps = p->sun_steps;
    tp.cone_mode = p->cone_mode;
    tp.cone_lanes = p->cone_lanes;
    tp.tan_half = (float)std::tan((double)p->cone_half_angle);
    tp.h0 = p->cone_initial_height;
    tp.rmin = p->cone_min_radius;
    tp.lod_offset = p->lod_offset;
    tp.down_scaling = p->down_scaling;
    tp.sigma = p->density_scale;
    tp.ambient = p->ambient;
    tp.cutoff = p->transmittance_cutoff;
    for (int a = 0; a < 3; ++a) tp.sun_color[a] = p->sun_color[a];
    double sx = sun_dir[0], sy = sun_dir[1], sz = sun_dir[2];
    double sn = std::sqrt(sx * sx + sy * sy + sz * sz);
    tp.sun[0] = (float)(sx / sn);
    tp.sun[1] = (float)(sy / sn);
    tp.sun[2] = (float)(sz / sn);
    tp.noise_seed = p->noise.seed;
    tp.noise_octaves = p->noise.octaves;
    tp.noise_freq = p->noise.frequency;
    tp.noise_lac = p->noise.lacunarity;
    tp.noise_gain = p->noise.gain;
    double norm = 0.0, amp = 1.0;
    for (int k = 0; k < p->noise.octaves; ++k) {
        norm += amp;
        amp *= (double)p->noise.gain;
    }
    tp.noise_inv_norm = norm > 0.0 ? (float)(1.0 / norm) : 1.0f;
    // the lattice offset as a world shift: (p * f + o) * lac^k = (p + o / f) * f * lac^k
    for (int a = 0; a < 3; ++a)
        tp.noise_shift[a] = p->noise.frequency != 0.f
                                ? (float)((double)p->noise.offset[a] / (double)p->noise.frequency)
                                : 0.f;
    memset(&tp.nt, 0, sizeof(tp.nt));
    return tp;
}

cg_status camera_of(const cg_camera* c, CamDesc& cam) {
    for (int a = 0; a < 3; ++a)
        CG_CHECK(std::isfinite(c->eye[a]) && std::isfinite(c->target[a]) &&
                     std::isfinite(c->up[a]),
                 CG_ERR_INVALID_ARGUMENT, "camera: non-finite vector");
    CG_CHECK(c->width >= 1 && c->height >= 1 && c->width <= 16384 && c->height <= 16384,
             CG_ERR_OUT_OF_RANGE, "camera: image %dx%d not in [1, 16384]^2", c->width,
             c->height);
    CG_CHECK(std::isfinite(c->fov_y_degrees) && c->fov_y_degrees > 0.f &&
                 c->fov_y_degrees < 180.f,
             CG_ERR_OUT_OF_RANGE, "camera: fov_y_degrees not in (0, 180)");
    double f[3], s[3], u[3];
    for (int a = 0; a < 3; ++a) f[a] = (double)c->target[a] - (double)c->eye[a];
    double fn = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    CG_CHECK(fn > 0.0, CG_ERR_INVALID_ARGUMENT, "camera: eye equals target");
    for (double& x : f) x /= fn;
    double up[3] = {c->up[0], c->up[1], c->up[2]};
    s[0] = f[1] * up[2] - up[1] * f[2];
    s[1] = f[2] * up[0] - up[2] * f[0];
    s[2] = f[0] * up[1] - up[0] * f[1];
    double sn = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    CG_CHECK(sn > 1e-12, CG_ERR_INVALID_ARGUMENT, "camera: up is parallel to the view direction");
    for (double& x : s) x /= sn;
    u[0] = s[1] * f[2] - f[1] * s[2];
    u[1] = s[2] * f[0] - f[2] * s[0];
    u[2] = s[0] * f[1] - f[0] * s[1];
    for (int a = 0; a < 3; ++a) {
        cam.eye[a] = c->eye[a];
        cam.f[a] = (float)f[a];
        cam.s[a] = (float)s[a];
        cam.u[a] = (float)u[a];
    }
    cam.tanh = (float)std::tan((double)c->fov_y_degrees * 3.14159265358979323846 / 360.0);
    cam.aspect = (float)c->width / (float)c->height;
    cam.W = c->width;
    cam.H = c->height;
    return CG_OK;
}

// Lattice tables for the render's noise parameters over the noise domain,
// rebuilt only when those change.  The domain is the volume's box; with a
// nonzero shift (wind) it is the box moved by the shift the tables were built
// for and widened by range/8 per side, so the tables (and the fBm volume) are
// rebuilt only when the shift has moved further than that.  Each octave covers
// floor(lo*f) - 1 .. floor(hi*f) + 2 per axis, f = frequency * lacunarity^o in
// FP32 as the kernel computes it; samples outside fall back to hashing (the
// same values).
cg_status ensure_noise(cg_context* ctx, const cg_volume* v, TraceParams& tp,
                              cudaStream_t s) {
    if (tp.noise_octaves <= 0) return CG_OK;
    float box[6] = {v->wmin[0], v->wmin[1], v->wmin[2], v->wmax[0], v->wmax[1], v->wmax[2]};
    const bool moving = tp.noise_shift[0] != 0.f || tp.noise_shift[1] != 0.f ||
                        tp.noise_shift[2] != 0.f;
    bool same = ctx->noise_valid && ctx->noise_seed == tp.noise_seed &&
                ctx->noise_octaves == tp.noise_octaves && ctx->noise_freq == tp.noise_freq &&
                ctx->noise_lac == tp.noise_lac && memcmp(ctx->noise_box, box, sizeof(box)) == 0 &&
                ctx->noise_moving == moving;
    if (same && moving)
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs((double)tp.noise_shift[a] - (double)ctx->noise_ref[a]) <=
                  (double)ctx->noise_margin[a]))
                same = false;
    if (!same) {
        double dom[6];
        for (int a = 0; a < 3; ++a) {
            const double m = moving ? 0.125 * ((double)box[3 + a] - (double)box[a]) : 0.0;
            const double ref = moving ? (double)tp.noise_shift[a] : 0.0;
            dom[a] = (double)box[a] + ref - m;
            dom[3 + a] = (double)box[3 + a] + ref + m;
        }
        NoiseTab nt{};
        long long total = 0;
        float f = tp.noise_freq;
        for (int o = 0; o < tp.noise_octaves; ++o) {
            nt.off[o] = (int)total;
            long long n = 1;
            for (int a = 0; a < 3; ++a) {
                double lo = std::floor(dom[a] * (double)f) - 1.0;
                double hi = std::floor(dom[3 + a] * (double)f) + 2.0;
                if (!(hi - lo < 4096.0) || !(lo > -1e9) || !(hi < 1e9)) {
                    n = -1;
                    break;
                }
                nt.lo[o][a] = (int)lo;
                nt.dim[o][a] = (int)(hi - lo) + 1;
                n *= nt.dim[o][a];
            }
            if (n < 0 || total + n > (64ll << 20)) {  // too large: hash on the fly
                total = -1;
                break;
            }
            total += n;
            f *= tp.noise_lac;
        }
        ctx->noise_valid = false;
        if (total > 0) {
            CG_CUDA(cudaStreamSynchronize(s));
            CG_CUDA(ctx->noise.ensure((size_t)total * 4));
            nt.tab = ctx->noise.as<const float>();
            tp.nt = nt;
            CG_LAUNCH(ctx, launch_noise_table(tp, ctx->noise.as<float>(), (int)total, s));
            // the same tables as 3D float textures (linear filter, unnormalised)
            release_noise_textures(ctx);
            for (int o = 0; o < tp.noise_octaves; ++o) {
                cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
                cudaExtent ext = make_cudaExtent(nt.dim[o][0], nt.dim[o][1], nt.dim[o][2]);
                CG_CUDA(cudaMalloc3DArray(&ctx->noise_arr[o], &fd, ext));
                cudaMemcpy3DParms cp = {};
                cp.srcPtr = make_cudaPitchedPtr(ctx->noise.as<float>() + nt.off[o],
                                                (size_t)nt.dim[o][0] * 4, nt.dim[o][0],
                                                nt.dim[o][1]);
                cp.dstArray = ctx->noise_arr[o];
                cp.extent = ext;
                cp.kind = cudaMemcpyDeviceToDevice;
                CG_CUDA(cudaMemcpy3DAsync(&cp, s));
                cudaResourceDesc rd = {};
                rd.resType = cudaResourceTypeArray;
                rd.res.array.array = ctx->noise_arr[o];
                cudaTextureDesc td = {};
                td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
                td.filterMode = cudaFilterModeLinear;
                td.readMode = cudaReadModeElementType;
                td.normalizedCoords = 0;
                CG_CUDA(cudaCreateTextureObject(&ctx->noise_tex[o], &rd, &td, nullptr));
                nt.tex[o] = ctx->noise_tex[o];
            }
            ctx->noise_tab = nt;
            ctx->noise_valid = true;
            ctx->noise_seed = tp.noise_seed;
            ctx->noise_octaves = tp.noise_octaves;
            ctx->noise_freq = tp.noise_freq;
            ctx->noise_lac = tp.noise_lac;
            memcpy(ctx->noise_box, box, sizeof(box));
            ctx->noise_moving = moving;
            for (int a = 0; a < 3; ++a) {
                ctx->noise_dom[a] = (float)dom[a];
                ctx->noise_dom[3 + a] = (float)dom[3 + a];
                ctx->noise_ref[a] = moving ? tp.noise_shift[a] : 0.f;
                ctx->noise_margin[a] = moving ? (float)(0.125 * ((double)box[3 + a] - (double)box[a])) : 0.f;
            }
        } else {
            memset(&ctx->noise_tab, 0, sizeof(ctx->noise_tab));
        }
    }
    tp.nt = ctx->noise_valid ? ctx->noise_tab : NoiseTab{};
    return CG_OK;
}

extern "C" cg_status cg_render(cg_context* ctx, const cg_volume* v, const cg_camera* cam,
                               const cg_render_params* params, float* rgba_out,
                               int out_on_device, void* stream) {
    NvtxRange nvtx_("cg_render");
    CG_CHECK(ctx && v && cam && params && rgba_out, CG_ERR_INVALID_ARGUMENT,
             "cg_render: null pointer");
    CG_CHECK(v->ctx == ctx, CG_ERR_INVALID_ARGUMENT, "cg_render: volume of another context");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_render: volume has not been voxelized");
    cg_status st = check_params(params);
    if (st != CG_OK) return st;
    CamDesc cd;
    st = camera_of(cam, cd);
    if (st != CG_OK) return st;
    MlpDev md;
    if (params->use_mlp) {
        st = mlp_device_for_render(params->mlp, v, params, md);
        if (st != CG_OK) return st;
    }
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t pixels = (size_t)cam->width * cam->height;
    float4* out = reinterpret_cast<float4*>(rgba_out);
    // host output: page-locked memory the device can address is written by
    // the pass that finishes the pixels (the image crosses the host link
    // while that kernel runs); any other host memory gets one copy at the end
    float4* dst = out;
    bool copy_back = false;
    if (!out_on_device) {
        CG_CUDA(ctx->image.ensure(pixels * 16));
        out = ctx->image.as<float4>();
        dst = out;
        copy_back = true;
        const bool finishes_directly =
            params->use_mlp || params->pipeline != CG_PIPELINE_DEFERRED;
        cudaPointerAttributes pa;
        if (finishes_directly && cudaPointerGetAttributes(&pa, rgba_out) == cudaSuccess &&
            pa.type == cudaMemoryTypeHost && pa.devicePointer && pa.device == ctx->device) {
            dst = reinterpret_cast<float4*>(pa.devicePointer);
            copy_back = false;
        }
        (void)cudaGetLastError();  // pageable memory may leave a query error behind
    }
    TraceParams tp = trace_params_of(params, v->sun_dir);
    stage_begin(ctx, s);
    st = ensure_noise(ctx, v, tp, s);
    if (st != CG_OK) return st;
    if (params->use_mlp) {
        st = ensure_textures(const_cast<cg_volume*>(v), s);
        if (st == CG_OK) st = ensure_fbm_volume(ctx, v, tp, s);
        if (st != CG_OK) return st;
        stage_mark(ctx, s, "textures");
    }
    const VolDesc vd = desc_of(v);
    if (params->use_mlp && params->pipeline == CG_PIPELINE_PERSISTENT &&
        32 * params->view_steps <= 0xFFFF) {
        // march, network and composite in one persistent kernel
        float* contrib = nullptr;
        uint2* steps = nullptr;
        st = ensure_render_slots(ctx, cam->width, cam->height, params->view_steps, contrib,
                                 steps);
        if (st != CG_OK) return st;
        CG_CUDA(cudaMemsetAsync(ctx->fallbacks.p, 0, 32, s));
        ctx->shaded_valid = true;
        CG_LAUNCH(ctx, launch_render_mlp_tc(vd, cd, tp, md, contrib, steps, dst,
                                            ctx->fallbacks.as<unsigned long long>(), s));
        stage_mark(ctx, s, "render_mlp");
    } else if (params->use_mlp || params->pipeline == CG_PIPELINE_DEFERRED) {
        // deferred: march records the contributing samples, shading resolves them
        SampleBuf sb;
        st = ensure_samples(ctx, cam->width, cam->height, params->view_steps, sb);
        if (st != CG_OK) return st;
        // the shading status block is cleared before the march, so that the
        // shading kernel directly follows it (a dependent launch)
        if (params->use_mlp) CG_CUDA(cudaMemsetAsync(ctx->fallbacks.p, 0, 32, s));
        CG_LAUNCH(ctx, launch_march(vd, cd, tp, sb, params->use_mlp != 0, s));
        stage_mark(ctx, s, "march");
        if (params->use_mlp) {
            ctx->shaded_valid = true;
            CG_LAUNCH(ctx, launch_shade_mlp_tc(vd, cd, tp, md, sb,
                                               ctx->fallbacks.as<unsigned long long>(), s));
            stage_mark(ctx, s, "shade_mlp");
            CG_LAUNCH(ctx, launch_accumulate(cd, tp, sb, dst, s));
            stage_mark(ctx, s, "accumulate");
        } else {
            CG_LAUNCH(ctx, launch_shade_exact(vd, cd, tp, sb, out, s));
            stage_mark(ctx, s, "shade_exact");
        }
    } else {
        CG_LAUNCH(ctx, launch_trace_fused(vd, cd, tp, dst, nullptr, s));
        stage_mark(ctx, s, "trace");
    }
    if (copy_back) CG_CUDA(cudaMemcpyAsync(rgba_out, out, pixels * 16, cudaMemcpyDeviceToHost, s));
    if (!out_on_device) CG_CUDA(cudaStreamSynchronize(s));
    return CG_OK;
}

extern "C" cg_status cg_render_stats(cg_context* ctx, const cg_volume* v, const cg_camera* cam,
                                     const cg_render_params* params, uint64_t counts[4]) {
    CG_CHECK(ctx && v && cam && params && counts, CG_ERR_INVALID_ARGUMENT,
             "cg_render_stats: null pointer");
    CG_CHECK(v->ctx == ctx, CG_ERR_INVALID_ARGUMENT, "cg_render_stats: volume of another context");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_render_stats: volume has not been voxelized");
    cg_status st = check_params(params);
    if (st != CG_OK) return st;
    CG_CHECK(!params->use_mlp, CG_ERR_UNSUPPORTED, "cg_render_stats: MLP surrogate not loaded");
    CamDesc cd;
    st = camera_of(cam, cd);
    if (st != CG_OK) return st;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t pixels = (size_t)cam->width * cam->height;
    CG_CUDA(ctx->image.ensure(pixels * 16));
    DevBuf cnt;
    CG_CUDA(cnt.ensure(64));
    TraceParams tp = trace_params_of(params, v->sun_dir);
    st = ensure_noise(ctx, v, tp, s);
    if (st != CG_OK) return st;
    cudaError_t e = cudaMemsetAsync(cnt.p, 0, 64, s);
    if (e == cudaSuccess)
        e = launch_trace_fused(desc_of(v), cd, tp, ctx->image.as<float4>(),
                               cnt.as<unsigned long long>(), s);
    unsigned long long h[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, cnt.p, 32, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cnt.release();
    if (e != cudaSuccess) return fail(CG_ERR_CUDA, "cg_render_stats: %s", cudaGetErrorString(e));
    ctx->launches++;
    for (int i = 0; i < 4; ++i) counts[i] = h[i];
    return CG_OK;
}

extern "C" cg_status cg_march_samples(cg_context* ctx, const cg_volume* v, const cg_camera* cam,
                                      const cg_render_params* params, float* positions,
                                      float* weights, int capacity, int* count) {
    CG_CHECK(ctx && v && cam && params && count && (capacity == 0 || (positions && weights)),
             CG_ERR_INVALID_ARGUMENT, "cg_march_samples: null pointer");
    CG_CHECK(capacity >= 0, CG_ERR_OUT_OF_RANGE, "cg_march_samples: capacity < 0");
    CG_CHECK(v->ctx == ctx, CG_ERR_INVALID_ARGUMENT, "cg_march_samples: volume of another context");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_march_samples: volume has not been voxelized");
    cg_status st = check_params(params);
    if (st != CG_OK) return st;
    CamDesc cd;
    st = camera_of(cam, cd);
    if (st != CG_OK) return st;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const size_t pixels = (size_t)cam->width * cam->height;
    CG_CUDA(ctx->image.ensure(pixels * 16));
    TraceParams tp = trace_params_of(params, v->sun_dir);
    st = ensure_noise(ctx, v, tp, s);
    if (st != CG_OK) return st;
    SampleBuf sb;
    st = ensure_samples(ctx, cam->width, cam->height, params->view_steps, sb);
    if (st != CG_OK) return st;
    CG_LAUNCH(ctx, launch_march(desc_of(v), cd, tp, sb, false, s));
    const size_t regions = (size_t)((cam->width + 15) / 16) * ((cam->height + 15) / 16) * 8;
    std::vector<unsigned> cnt(regions);
    CG_CUDA(cudaMemcpyAsync(cnt.data(), sb.count, regions * 4, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    size_t total = 0;
    std::vector<float4> tmp;
    for (size_t r = 0; r < regions; ++r) {
        if (!cnt[r]) continue;
        tmp.resize(cnt[r]);
        CG_CUDA(cudaMemcpy(tmp.data(), sb.pos_w + r * (size_t)sb.capacity, cnt[r] * 16,
                           cudaMemcpyDeviceToHost));
        for (unsigned i = 0; i < cnt[r]; ++i, ++total) {
            if (total >= (size_t)capacity) continue;
            positions[3 * total] = tmp[i].x;
            positions[3 * total + 1] = tmp[i].y;
            positions[3 * total + 2] = tmp[i].z;
            weights[total] = tmp[i].w;
        }
    }
    *count = (int)std::min(total, (size_t)0x7FFFFFFF);
    return CG_OK;
}

extern "C" cg_status cg_trace_cones(const cg_volume* v, const float* positions, int n,
                                    const float direction[3], const cg_render_params* params,
                                    float* out, int on_device, void* stream) {
    CG_CHECK(v && direction && params && (n == 0 || (positions && out)),
             CG_ERR_INVALID_ARGUMENT, "cg_trace_cones: null pointer");
    CG_CHECK(n >= 0, CG_ERR_OUT_OF_RANGE, "cg_trace_cones: n < 0");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_trace_cones: volume has not been voxelized");
    cg_status st = check_params(params);
    if (st != CG_OK) return st;
    double dn = std::sqrt((double)direction[0] * direction[0] + (double)direction[1] * direction[1] +
                          (double)direction[2] * direction[2]);
    CG_CHECK(std::isfinite(dn) && dn > 0.0, CG_ERR_INVALID_ARGUMENT,
             "cg_trace_cones: direction must be finite and non-zero");
    if (n == 0) return CG_OK;
    cg_context* ctx = v->ctx;
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    TraceParams tp = trace_params_of(params, direction);
    const float* dpos = positions;
    float* dout = out;
    DevBuf tmp;
    if (!on_device) {
        CG_CUDA(tmp.ensure((size_t)n * 16));
        float* base = tmp.as<float>();
        CG_CUDA(cudaMemcpyAsync(base, positions, (size_t)n * 12, cudaMemcpyHostToDevice, s));
        dpos = base;
        dout = base + (size_t)n * 3;
    }
    cudaError_t e = launch_trace_cones(desc_of(v), tp, dpos, n, dout, s);
    if (e != cudaSuccess) {
        tmp.release();
        return fail(CG_ERR_CUDA, "launch_trace_cones: %s", cudaGetErrorString(e));
    }
    ctx->launches++;
    if (!on_device) {
        e = cudaMemcpyAsync(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        tmp.release();
        if (e != cudaSuccess) return fail(CG_ERR_CUDA, "cg_trace_cones: %s", cudaGetErrorString(e));
    }
    return CG_OK;
}

// ---------------------------------------------------------------------------
// readback
// ---------------------------------------------------------------------------
extern "C" cg_status cg_volume_get_info(const cg_volume* v, cg_volume_info* info) {
    CG_CHECK(v && info, CG_ERR_INVALID_ARGUMENT, "cg_volume_get_info: null pointer");
    memset(info, 0, sizeof(*info));
    info->dimension = v->D;
    info->mips = v->L;
    info->format = v->fmt;
    info->board_count = v->n;
    for (int a = 0; a < 3; ++a) {
        info->world_min[a] = v->wmin[a];
        info->world_max[a] = v->wmax[a];
    }
    for (int l = 0; l < 16; ++l) {
        info->level_dim[l] = l < v->L ? v->dims[l] : 0;
        info->level_offset[l] = v->offs[l];
    }
    info->bytes_per_voxel = v->fmt == CG_FORMAT_RGBA32F ? 16 : 4;
    info->pyramid_bytes = v->total * info->bytes_per_voxel;
    return CG_OK;
}

static cg_status sync_volume(const cg_volume* v) {
    CG_CUDA(cudaSetDevice(v->ctx->device));
    CG_CUDA(cudaDeviceSynchronize());  // voxelize may have run on a caller's stream
    return CG_OK;
}

// The integer coverage (count, Q16.16 density) of the last voxelize, computed
// on demand by the coverage-only splat (voxelize itself stores only the
// pyramid).
static cg_status ensure_coverage(const cg_volume* cv) {
    cg_volume* v = const_cast<cg_volume*>(cv);
    if (v->cov_gen == v->gen) return CG_OK;
    CG_CHECK(!v->boards_dirty, CG_ERR_NOT_READY,
             "coverage: the billboards changed since the last voxelize; voxelize again");
    cg_status st = sync_volume(v);
    if (st != CG_OK) return st;
    cudaStream_t s = v->ctx->stream;
    Bins bins = v->bins;
    bins.count = v->bcount.as<uint32_t>();
    bins.offset = v->boff.as<uint32_t>();
    bins.cursor = v->bcursor.as<uint32_t>();
    bins.list = v->blist.as<uint32_t>();
    bins.dirty = v->bdirty.as<uint8_t>();
    bins.hl = nullptr;  // the coverage-only splat reads no mask
    CG_LAUNCH(v->ctx, launch_splat(boards_of(v), bins, v->mask.as<uint8_t>(), desc_of(v), v->pyr.p,
                                   v->count.as<uint32_t>(), v->dq.as<uint32_t>(), 0,
                                   raw_of(v), true, s));
    CG_CUDA(cudaStreamSynchronize(s));
    v->cov_gen = v->gen;
    return CG_OK;
}

extern "C" cg_status cg_volume_read_level(const cg_volume* v, int level, void* dst,
                                          size_t dst_bytes) {
    CG_CHECK(v && dst, CG_ERR_INVALID_ARGUMENT, "cg_volume_read_level: null pointer");
    CG_CHECK(level >= 0 && level < v->L, CG_ERR_OUT_OF_RANGE,
             "cg_volume_read_level: level %d not in [0, %d)", level, v->L);
    const size_t bpv = v->fmt == CG_FORMAT_RGBA32F ? 16 : 4;
    const size_t n = (size_t)v->dims[level] * v->dims[level] * v->dims[level];
    CG_CHECK(dst_bytes >= n * bpv, CG_ERR_OUT_OF_RANGE,
             "cg_volume_read_level: buffer %zu B < %zu B", dst_bytes, n * bpv);
    cg_status st = sync_volume(v);
    if (st != CG_OK) return st;
    CG_CUDA(cudaMemcpy(dst, reinterpret_cast<const char*>(v->pyr.p) + v->offs[level] * bpv,
                       n * bpv, cudaMemcpyDeviceToHost));
    return CG_OK;
}

extern "C" cg_status cg_volume_read_coverage(const cg_volume* v, uint32_t* count,
                                             uint32_t* density_q16) {
    CG_CHECK(v && count && density_q16, CG_ERR_INVALID_ARGUMENT,
             "cg_volume_read_coverage: null pointer");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_volume_read_coverage: not voxelized");
    cg_status st = ensure_coverage(v);
    if (st != CG_OK) return st;
    const size_t n0 = (size_t)v->D * v->D * v->D;
    CG_CUDA(cudaMemcpy(count, v->count.p, n0 * 4, cudaMemcpyDeviceToHost));
    CG_CUDA(cudaMemcpy(density_q16, v->dq.p, n0 * 4, cudaMemcpyDeviceToHost));
    return CG_OK;
}

extern "C" cg_status cg_volume_read_sun_map(const cg_volume* v, uint64_t* keys, float* positions) {
    CG_CHECK(v && keys && positions, CG_ERR_INVALID_ARGUMENT,
             "cg_volume_read_sun_map: null pointer");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_volume_read_sun_map: not voxelized");
    cg_status st = sync_volume(v);
    if (st != CG_OK) return st;
    const size_t t = (size_t)v->mapW * v->mapH;
    CG_CUDA(cudaMemcpy(keys, v->keys.p, t * 8, cudaMemcpyDeviceToHost));
    CG_CUDA(cudaMemcpy(positions, v->posmap.p, t * 16, cudaMemcpyDeviceToHost));
    return CG_OK;
}

extern "C" cg_status cg_volume_read_highlight(const cg_volume* v, uint8_t* mask) {
    CG_CHECK(v && mask, CG_ERR_INVALID_ARGUMENT, "cg_volume_read_highlight: null pointer");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_volume_read_highlight: not voxelized");
    cg_status st = sync_volume(v);
    if (st != CG_OK) return st;
    CG_CUDA(cudaMemcpy(mask, v->mask.p, (size_t)v->D * v->D * v->D, cudaMemcpyDeviceToHost));
    return CG_OK;
}

extern "C" cg_status cg_volume_active_voxels(const cg_volume* v, uint64_t* active) {
    CG_CHECK(v && active, CG_ERR_INVALID_ARGUMENT, "cg_volume_active_voxels: null pointer");
    CG_CHECK(v->voxelized, CG_ERR_NOT_READY, "cg_volume_active_voxels: not voxelized");
    cg_status st = ensure_coverage(v);
    if (st != CG_OK) return st;
    cudaStream_t s = v->ctx->stream;
    unsigned long long* d = const_cast<cg_volume*>(v)->scratch.as<unsigned long long>();
    CG_CUDA(cudaMemsetAsync(d, 0, 8, s));
    CG_LAUNCH(v->ctx, launch_count_active(v->count.as<uint32_t>(), v->mask.as<uint8_t>(),
                                          (size_t)v->D * v->D * v->D, d, s));
    unsigned long long h = 0;
    CG_CUDA(cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    *active = h;
    return CG_OK;
}

extern "C" cg_status cg_image_error_stats(cg_context* ctx, const float* image,
                                          const void* reference, int reference_is_f64,
                                          uint64_t pixels, int on_device, double out[10],
                                          void* stream) {
    CG_CHECK(ctx && image && reference && out, CG_ERR_INVALID_ARGUMENT,
             "cg_image_error_stats: null pointer");
    CG_CHECK(pixels > 0, CG_ERR_INVALID_ARGUMENT, "cg_image_error_stats: no pixels");
    CG_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = pick_stream(ctx, stream);
    const size_t ref_bytes = (size_t)pixels * 4 * (reference_is_f64 ? 8 : 4);
    const float* a = image;
    const void* ref = reference;
    if (!on_device) {
        CG_CUDA(ctx->stats_a.ensure((size_t)pixels * 16));
        CG_CUDA(ctx->stats_ref.ensure(ref_bytes));
        CG_CUDA(cudaMemcpyAsync(ctx->stats_a.p, image, (size_t)pixels * 16,
                                cudaMemcpyHostToDevice, s));
        CG_CUDA(cudaMemcpyAsync(ctx->stats_ref.p, reference, ref_bytes, cudaMemcpyHostToDevice,
                                s));
        a = ctx->stats_a.as<const float>();
        ref = ctx->stats_ref.p;
    }
    CG_CUDA(ctx->stats_scratch.ensure(err_stats_scratch_bytes() + 8 * sizeof(double)));
    double* part = ctx->stats_scratch.as<double>();
    double* dres = part + (err_stats_scratch_bytes() / sizeof(double));
    CG_LAUNCH(ctx, launch_err_stats(reinterpret_cast<const float4*>(a), ref, reference_is_f64,
                                    (size_t)pixels, part, dres, s));
    ctx->launches++;  // the final reduction
    double h[8];
    CG_CUDA(cudaMemcpyAsync(h, dres, sizeof(h), cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    double mx = 0, ss = 0;
    for (int c = 0; c < 4; ++c) {
        out[c] = h[c];
        out[4 + c] = std::sqrt(h[4 + c] / (double)pixels);
        mx = h[c] > mx ? h[c] : mx;
        ss += h[4 + c];
    }
    out[8] = mx;
    out[9] = std::sqrt(ss / (4.0 * (double)pixels));
    return CG_OK;
}

extern "C" cg_status cg_volume_set_occupancy_brick(cg_volume* v, int brick) {
    CG_CHECK(v, CG_ERR_INVALID_ARGUMENT, "cg_volume_set_occupancy_brick: volume is NULL");
    CG_CHECK(brick == 4 || brick == 8 || brick == 16, CG_ERR_OUT_OF_RANGE,
             "cg_volume_set_occupancy_brick: brick %d not in {4, 8, 16}", brick);
    if (brick == v->occ_brick) return CG_OK;
    CG_CUDA(cudaSetDevice(v->ctx->device));
    CG_CUDA(cudaDeviceSynchronize());
    set_occ_layout(v, brick);
    if (v->voxelized) {
        // rebuild the brick grids (and the occupied box) from the raw cells of
        // the last voxelize
        const VolDesc vd = desc_of(v);
        CG_CUDA(cudaMemsetAsync(const_cast<int*>(vd.occ_box), 0, 6 * sizeof(int),
                                v->ctx->stream));
        CG_LAUNCH(v->ctx, launch_occ_dilate(vd, raw_of(v), v->occ.as<uint8_t>() + v->raw_total,
                                            v->occ_total, v->ctx->stream));
        CG_CUDA(cudaStreamSynchronize(v->ctx->stream));
    }
    return CG_OK;
}

