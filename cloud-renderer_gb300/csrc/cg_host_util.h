// cg_host_util.h -- host-side internals shared by the C-ABI translation units:
// error reporting, device/host buffers and the context and volume objects.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "cg_internal.h"
#include "cloudgb.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
cg_status fail(cg_status s, const char* fmt, ...);

#define CG_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(e_ == cudaErrorMemoryAllocation ? CG_ERR_OUT_OF_MEMORY : CG_ERR_CUDA, \
                        "%s: %s", #call, cudaGetErrorString(e_));                          \
    } while (0)

#define CG_CHECK(cond, status, ...)                  \
    do {                                             \
        if (!(cond)) return fail(status, __VA_ARGS__); \
    } while (0)

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, want ? want : 16);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

struct HostBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want) {
        if (want <= bytes && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMallocHost(&p, want ? want : 16);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

struct cg_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    // voxelize: the sun-view pass (sun map + highlights) runs on `side`,
    // concurrently with the brick binning, forked and joined by two events
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaEvent_t clear_ev = nullptr;  // voxelize: the mask cleared (on the caller's stream)
    uint64_t launches = 0;
    int refs = 1;  // the caller's handle + one per volume / model created on it
    bool shaded_valid = false;  // the status words hold a surrogate render's counters
    // optional per-stage CUDA-event timing of voxelize/render calls
    bool timing = false;
    int n_marks = 0;
    cudaEvent_t marks[32] = {};
    char mark_names[32][24] = {};
    DevBuf image;  // render target when the caller passes a host pointer
    // hash-noise lattice tables of the last (noise parameters, world box)
    DevBuf noise;
    bool noise_valid = false;
    uint32_t noise_seed = 0;
    int noise_octaves = 0;
    float noise_freq = 0, noise_lac = 0, noise_box[6] = {0, 0, 0, 0, 0, 0};
    // noise domain the tables cover; for a moving (wind) shift: the shift they
    // were built around and how far it may move before a rebuild
    bool noise_moving = false;
    float noise_dom[6] = {0, 0, 0, 0, 0, 0};
    float noise_ref[3] = {0, 0, 0}, noise_margin[3] = {0, 0, 0};
    NoiseTab noise_tab{};
    // deferred renderer: recorded view samples and the MLP fallback counter
    DevBuf samples_pw, samples_gl, samples_cnt, samples_c, samples_alpha;
    DevBuf fallbacks;  // surrogate render status (see launch_shade_mlp_tc)
    DevBuf stats_scratch, stats_a, stats_ref;  // cg_image_error_stats staging
    // batch render: launch shape, descriptors (host, pinned staging, device
    // descriptors + tile counter)
    cg_trace_config trace_cfg{1, 1, 0};
    std::vector<BatchView> batch_host;
    HostBuf batch_pinned;
    DevBuf batch_dev;
    // compat render: noise map (green, alpha) of compat_seed, per-board tile
    // rectangles and keys, per-tile counts / offsets / cursors, the lists
    DevBuf compat_noise;
    bool compat_noise_valid = false;
    uint32_t compat_seed = 0;
    DevBuf compat_rect, compat_key, compat_tiles, compat_list;
    HostBuf compat_total;
    // noise lattice tables as 3D float textures (surrogate renderer)
    cudaArray_t noise_arr[CG_MAX_LEVELS] = {};
    cudaTextureObject_t noise_tex[CG_MAX_LEVELS] = {};
    // the fBm sampled on a grid (surrogate renderer), valid for the current tables
    cudaArray_t fbm_arr = nullptr;
    cudaSurfaceObject_t fbm_surf = 0;
    cudaTextureObject_t fbm_tex = 0;
    int fbm_res = 0;
    bool fbm_valid = false;
};

void release_noise_textures(cg_context* ctx);
cg_status ensure_fbm_volume(cg_context* ctx, const cg_volume* v, TraceParams& tp, cudaStream_t s);

struct cg_volume {
    cg_context* ctx = nullptr;
    int D = 0, L = 0, fmt = 0;
    float pos[3] = {0, 0, 0}, b0 = 0, b1 = 0;
    float wmin[3], wmax[3], range[3];
    int dims[CG_MAX_LEVELS];
    size_t offs[CG_MAX_LEVELS];
    size_t total = 0;
    DevBuf pyr, count, dq, mask;
    // boards
    int n = 0;
    size_t pairs = 0;
    // board records in one allocation, uploaded with one copy: float4 centre +
    // radius, int4 Q20 centre + radius, u64 ball threshold, u32 Q16 density,
    // u8 culled (offsets 0, 16n, 32n, 40n, 44n)
    DevBuf boards;
    float4* cwr = nullptr;
    int4* q = nullptr;
    uint64_t* thr = nullptr;
    uint32_t* dqb = nullptr;
    uint8_t* culled = nullptr;
    HostBuf h_stage;
    Bins bins{};
    DevBuf bcount, boff, bcursor, blist, bdirty;
    DevBuf bhl;  // per-brick highlight flags of the current voxelize
    // sun map
    int mapW = 0, mapH = 0;
    DevBuf keys, posmap;
    bool voxelized = false;
    SunFrame frame{};
    float sun_dir[3] = {0, 1, 0};
    DevBuf scratch;  // small scalars (active voxel count)
    DevBuf occ;      // raw occupancy cells (OccRaw), then the brick grids (VolDesc)
    int raw_nb[CG_MAX_LEVELS];
    int raw_off[CG_MAX_LEVELS];
    int raw_total = 0;
    int occ_brick = 4;
    int occ_nb[CG_MAX_LEVELS];
    int occ_off[CG_MAX_LEVELS];
    int occ_total = 0;
    // half2 texture copies of the levels for the surrogate renderer, rebuilt
    // lazily after each voxelize (gen counts voxelizations)
    cudaArray_t tex_arr[CG_MAX_LEVELS] = {};
    cudaSurfaceObject_t tex_surf[CG_MAX_LEVELS] = {};
    cudaTextureObject_t tex_obj[CG_MAX_LEVELS] = {};
    long long gen = 0, tex_gen = -1;
    long long cov_gen = -1;  // voxelization whose integer coverage is in count / dq
    bool boards_dirty = false;  // billboards replaced since the last voxelize
    // cross-stream order of board uploads (context stream) and voxelizes (any
    // stream): boards_ready follows the last upload's copies, boards_read the
    // last voxelize that read the board buffers (direct or graph replay)
    cudaEvent_t boards_ready = nullptr, boards_read = nullptr;
    bool ready_pending = false, read_pending = false;
};

cg_status ensure_textures(cg_volume* v, cudaStream_t s);

VolDesc desc_of(const cg_volume* v);
// Byte offset of the level-0 occupied box in the volume's occupancy buffer.
size_t occ_box_offset(int raw_total);
OccRaw raw_of(const cg_volume* v);
void set_occ_layout(cg_volume* v, int brick);
BoardsDev boards_of(const cg_volume* v);
cg_status check_params(const cg_render_params* p);
TraceParams trace_params_of(const cg_render_params* p, const float sun_dir[3]);
cg_status camera_of(const cg_camera* c, CamDesc& cam);
cg_status ensure_noise(cg_context* ctx, const cg_volume* v, TraceParams& tp, cudaStream_t s);
cudaStream_t pick_stream(cg_context* ctx, void* stream);
void context_retain(cg_context* ctx);
void context_release(cg_context* ctx);
// Stage timing: stage_begin records the start event of a call, stage_mark the
// end of a named stage (no-ops unless timing is on).
void stage_begin(cg_context* ctx, cudaStream_t s);
void stage_mark(cg_context* ctx, cudaStream_t s, const char* name);

// NVTX range over a scope: profilers (ncu --nvtx, nsys) attribute the launches
// enqueued inside it to `name`.  Without an attached tool the calls return at
// once (NVTX v3 is header-only and loads a tool library only when one is set).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// cg_mlp.cpp
struct SampleBuf;
struct MlpDev;
cg_status ensure_samples(cg_context* ctx, int width, int height, int view_steps, SampleBuf& sb);
// Contribution slots and step tables of the fused surrogate renderer
// (launch_render_mlp_tc's layout), in the context's sample buffers.
cg_status ensure_render_slots(cg_context* ctx, int width, int height, int view_steps,
                              float*& contrib, uint2*& steps);
cg_status mlp_device_for_render(const cg_mlp* m, const cg_volume* v, const cg_render_params* p,
                                MlpDev& md);

#define CG_LAUNCH(ctx, expr)                                                          \
    do {                                                                              \
        cudaError_t e_ = (expr);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(CG_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_));        \
        (ctx)->launches++;                                                            \
    } while (0)
