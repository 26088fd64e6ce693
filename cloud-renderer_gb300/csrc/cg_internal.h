// cg_internal.h -- structures shared by the host library and the kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "cg_check.cuh"

#define CG_MAX_LEVELS 16
#define CG_Q20 1048576LL
#define CG_HALF_Q20 524288LL
#define CG_KEY_EMPTY 0xFFFFFFFFFFFFFFFFULL
#define CG_NO_SLOT 0xFFFFFFFFu
#define CG_MAX_SUN_STEPS 64
#define CG_BRICK 8           // splat brick edge (voxels)
#define CG_FUSED_MIPS 3      // levels produced inside the splat kernel
#define CG_SPLAT_CHUNK 256   // boards staged in shared memory per pass

// ---- programmatic dependent launch: a kernel launched with
// launch_dependent() may start while the kernel before it on the stream is
// still running; it runs its independent prologue, then grid_dep_wait()
// blocks until that kernel has completed and its memory is visible.  A
// kernel calls grid_dep_trigger() once its dependent may be scheduled (else
// at its exit).  Both are no-ops for an ordinary launch.
#ifdef __CUDACC__
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                    cudaStream_t st, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}
#endif

// Sun-view frame: lookAt basis + ortho window (Sun::update, Sun.hpp:26-43).
struct SunFrame {
    float eye[3], right[3], up[3], fwd[3], t[3];
    float lo, hi, near_z, clip;
    int W, H;
};

// Pyramid description passed by value to kernels.
//
// Occupancy: for every level l a grid of occ_nb[l]^3 bytes, one per brick of
// B^3 level-l texels, B = 1 << occ_shift (4, 8 or 16; a texel (x,y,z) is in
// brick (x,y,z) >> occ_shift).  A byte is 1 when the brick or one of its 26
// neighbours holds a voxel with density R > 0.  Because the mips are means of
// non-negative values, a trilinear footprint whose brick reads 0 has R = 0
// exactly, so samplers may skip it.
struct VolDesc {
    int D, L, fmt;
    int dims[CG_MAX_LEVELS];
    long long offs[CG_MAX_LEVELS];  // voxels
    float lsc[CG_MAX_LEVELS];       // (float)dims[l] / (float)D, level-0 voxel -> level-l texel
    float wmin[3], range[3];
    const void* pyr;                // float4* (RGBA32F) or uint32_t* (BF16_FP16)
    const uint8_t* occ;             // occupancy grids, concatenated by level
    // level-0 box of the occupied (dilated) bricks, in level-0 voxels:
    // [0..2] = D - lo, [3..5] = hi (exclusive); lo >= hi when nothing is occupied
    const int* occ_box;
    int occ_shift;
    int occ_nb[CG_MAX_LEVELS];
    int occ_off[CG_MAX_LEVELS];
    // hardware-filtered half2 (density, light) copies of the levels for the
    // surrogate renderer (cudaTextureObject_t; 0 when not built)
    unsigned long long tex[CG_MAX_LEVELS];
    // surfaces of the same arrays (cudaSurfaceObject_t): when set, voxelize
    // writes each stored voxel there too, so the copies never need a pass
    unsigned long long surf[CG_MAX_LEVELS];
    // voxels of all levels and bytes of all occupancy grids (the bounds of
    // the bounds-check build)
    long long nvox;
    int occ_total;
};

// Hash-noise lattice values tabulated per octave over the world box: octave
// k covers lattice points lo[k] + [0, dim[k]) per axis, row-major x fastest,
// starting at off[k] in the table.  Values equal the on-the-fly hash bit for
// bit; points outside a table fall back to hashing.
struct NoiseTab {
    const float* tab;
    int off[CG_MAX_LEVELS];
    int lo[CG_MAX_LEVELS][3];
    int dim[CG_MAX_LEVELS][3];
    // the same tables as 3D float textures for the surrogate renderer (0 = none)
    unsigned long long tex[CG_MAX_LEVELS];
    // the whole fBm sampled on a fbm_res^3 grid of texel centres over the noise
    // domain (surrogate renderer; 8 texels per finest lattice cell): noise
    // coordinate q sits at texel coordinate (q - fbm_org) * fbm_sc
    unsigned long long fbm_tex;
    int fbm_res;
    float fbm_org[3], fbm_sc[3];
};

// Camera in FP32 for the trace kernels.
struct CamDesc {
    float eye[3], f[3], s[3], u[3];
    float tanh, aspect;
    int W, H;
};

// Render parameters resolved for the device.
struct TraceParams {
    int view_steps, sun_steps, cone_mode;
    int cone_lanes;  // warp-cooperative sun cones in the fused trace (0: off)
    float tan_half, h0, rmin, lod_offset, down_scaling;
    float sigma, ambient, cutoff;
    float sun_color[3];
    float sun[3];   // unit direction toward the sun
    uint32_t noise_seed;
    int noise_octaves;
    float noise_freq, noise_lac, noise_gain, noise_inv_norm;
    float noise_shift[3];  // world shift of the noise domain (offset / frequency)
    NoiseTab nt;
};

// Sun-cone schedule.  The cone's heights and radii do not depend on the
// volume, so they are computed once per launch on the host (FP64) and read
// from the kernel parameters: step i samples at v + h[i] * s with lod l0[i] +
// frac[i] and weight w[i] (r_i * voxel_world for the transmittance cone,
// i / (steps * downScaling) for the reference cone).
struct ConeSchedule {
    int steps;
    int mode;         // 0 transmittance (border 0), 1 reference (clamp to edge)
    float edge;       // break when a sample lies further than this outside the box
    float h[CG_MAX_SUN_STEPS];
    float w[CG_MAX_SUN_STEPS];
    float frac[CG_MAX_SUN_STEPS];
    unsigned char l0[CG_MAX_SUN_STEPS];
};

// Per-board device arrays (SoA).
struct BoardsDev {
    int n;
    const float4* cwr;      // world centre xyz, radius w
    const int4* q;          // Q20 voxel-space centre xyz, radius w (coverage)
    const uint64_t* thr;    // squared-radius threshold, Q40
    const uint32_t* dq;     // Q16.16 density
    const uint8_t* culled;  // 1 = no coverage contribution
};

// Raw occupancy written by the splat: per level, one byte per 4^3 texels
// (nb[l] = ceil(dims[l] / 4)), 1 when a voxel of the cell has R > 0.
struct OccRaw {
    uint8_t* raw;
    int nb[CG_MAX_LEVELS];
    int off[CG_MAX_LEVELS];
};

struct Bins {
    int nbx, nby, nbz, nbricks;
    uint32_t* count;   // nbricks
    uint32_t* offset;  // nbricks + 1
    uint32_t* cursor;  // nbricks
    uint32_t* list;    // pairs
    // per brick: 1 when its level-0 voxels (and fused levels 1-3) may hold
    // non-zero values from an earlier voxelize; a brick without boards or
    // highlights whose flag is 0 is already all zero and is not rewritten
    uint8_t* dirty;    // nbricks
    // per brick: 1 when a highlight store of this voxelize marked one of its
    // voxels (written by the highlight pass; NULL: the splat reads the mask)
    const uint8_t* hl;
};

// ---- deferred renderer ----------------------------------------------------
// View samples recorded by the march pass, one region of `capacity` slots per
// warp (8x4 pixel tile).  pos_w = level-0 voxel position + weight T*alpha;
// light_lane = light channel G + the pixel's lane (int bits).
struct SampleBuf {
    float4* pos_w;
    float2* light_lane;
    float* contrib;   // per slot: the sample's shaded contribution (surrogate path)
    unsigned* count;  // samples per region
    // flat order (written by the march): each march CTA's 8 regions occupy a
    // contiguous range, padded to 32-sample chunks; slot_of[i] = slot
    // (region * capacity + j) of flat row i, or CG_NO_SLOT for padding;
    // *flat_total = padded total (zeroed before the march)
    unsigned* slot_of;
    unsigned* flat_total;
    uint2* steps;     // per region, per emitting step: (first slot, lane ballot)
    unsigned* nsteps; // emitting steps per region
    float* alpha;     // per pixel (row-major, W x H): 1 - T after the march
    int capacity;     // 32 * view_steps
    unsigned long long nslots;  // regions * capacity
};

// ---- MLP surrogate ----------------------------------------------------------
#define MLP_IN 16
#define MLP_H 64
// hidden layers: 1, 2 or 3 of width 64 (a model's depth is fixed when it is
// created); the parameter vector always has room for three, and the blocks of
// the layers a model does not use stay zero and are never updated
#define MLP_MAX_LAYERS 3
#define MLP_DEFAULT_LAYERS 3
// flat FP32 parameter vector: W stored [out][in]
#define MLP_W1 0
#define MLP_B1 1024
#define MLP_W2 1088
#define MLP_B2 5184
#define MLP_W3 5248
#define MLP_B3 9344
#define MLP_W4 9408
#define MLP_B4 9472
#define MLP_NPARAM 9473
// FP16 weight image: W1 [64][16], W2 [64][64], W3 [64][64], W4 [8][64] (rows 1-7 zero)
#define MLP_H_W1 0
#define MLP_H_W2 1024
#define MLP_H_W3 5120
#define MLP_H_W4 9216
#define MLP_NHALF 9728

// Feature geometry and normalisation of a trained model.
//   f[3i+k] = R at level lb+i (clamped to the pyramid) sampled at
//             v + (h0 + (k + 0.5) * 2^(lb+i)) * s,   i = 0..3, k = 0..2
//   f[12..14] = v / D,  f[15] = s.y (cosine of the sun's zenith angle)
// Inputs are normalised x = (f - mu) * inv_sd; the output y gives
// tau = tau_scale * softplus(y).  Samples with a feature outside
// [fmin, fmax] fall back to the exact cone.
// Biases and the output row by value (kernel parameters, so that unrolled
// code reads them as constant operands): hb = (b1 | b2 | b3) / 2 for the
// half-scaled hidden layers of the inference kernel, w4 = W4 row 0 as
// FP16-rounded floats, b4 the output bias.
struct MlpConsts {
    float hb[3 * MLP_H];
    float w4[MLP_H];
    float b4;
};

struct MlpDev {
    const float* params;  // FP32 master (biases read from here)
    const __half* w16;    // FP16 weight image
    float mu[MLP_IN], inv_sd[MLP_IN], fmin[MLP_IN], fmax[MLP_IN];
    float tau_scale;
    float h0;
    int lb;
    int layers;           // hidden layers in use (1 .. MLP_MAX_LAYERS)
    MlpConsts k;          // copy of the current biases (for inference)
};

// Parameters [lo, hi) of the hidden layers a model of `layers` does not use
// (W2 .. b3 for one layer, W3 .. b3 for two, none for three).
inline void mlp_frozen_range(int layers, int& lo, int& hi) {
    lo = layers <= 1 ? MLP_W2 : (layers == 2 ? MLP_W3 : 0);
    hi = layers >= MLP_MAX_LAYERS ? 0 : MLP_W4;
}

// Feature-tap geometry of a (model, volume) pair, precomputed on the host:
// tap 3i+k reads level l_i (tex[i]) at texel coordinate v * sc[i] + dsc[3i+k] * s.
struct FeatGeom {
    float dsc[12];
    float sc[4];
    unsigned long long tex[4];
    float invD;
};

inline FeatGeom feat_geom(const VolDesc& vd, const MlpDev& m) {
    FeatGeom g;
    for (int i = 0; i < 4; ++i) {
        const int lv = m.lb + i;
        const int l = lv < 0 ? 0 : (lv > vd.L - 1 ? vd.L - 1 : lv);
        const float sc = (float)vd.dims[l] / (float)vd.D;
        const float span = (float)(1 << lv);
        for (int k = 0; k < 3; ++k) g.dsc[3 * i + k] = (m.h0 + ((float)k + 0.5f) * span) * sc;
        g.sc[i] = sc;
        g.tex[i] = vd.tex[l];
    }
    g.invD = 1.f / (float)vd.D;
    return g;
}

struct AdamArgs {
    const float* partial;
    int nparts;
    float inv_batch;
    float* params;
    __half* w16;
    float* m;
    float* v;
    float lr, beta1, beta2, eps;
    int* step;           // device step counter (NULL: single evaluation)
    unsigned* ticket;    // last-CTA detection
    float* grad_out;     // non-NULL: write the reduced gradient, no update
    float* loss_out;     // mean loss; index step - loss_base (or 0)
    int loss_slot_by_step;
    int loss_base;
    // the training kernel's status word (NULL: none); when it is non-zero the
    // partials may be stale or half-written, so no update is made and the
    // step counter does not advance
    const unsigned long long* status;
    // parameters of unused hidden layers (mlp_frozen_range): no partials are
    // written for them; their gradient reads 0 and they are never updated
    int frozen_lo, frozen_hi;
};

struct TrainArgs {
    const float* feat;  // [N][16] raw features
    const float* tau;   // [N] exact optical depth
    long long N;
    unsigned long long perm_mul;  // multiplier coprime with N
    float mu[16], inv_sd[16];
    float tau_scale, sigma;
    const float* params;
    const __half* w16;
    float* partial;   // [ctas][MLP_NPARAM + 1]
    const int* step;  // device step counter (NULL: 0)
    int layers;       // hidden layers (1 .. MLP_MAX_LAYERS)
    int batch;
    int sequential;   // 1: rows offset + r (gradient evaluation), padding past N
    long long offset;
    // tensor-core status word (zeroed by the host before the steps): bit 0 =
    // a bounded wait ran out, bit 1 = the drain after it ran out as well,
    // bit 2 = the fused optimiser's grid barrier ran out
    unsigned long long* status;
    unsigned long long wait_ns;  // limit of every mbarrier wait
    // failure-detection check only: thread 0 issues no MMA and no commit, so
    // the layer barrier is never completed and the first wait must run out
    int stall;
    // optimiser in the same launch (cooperative: every CTA resident).  After
    // its partials each CTA meets the others at a bounded grid barrier on
    // grid_bar (an arrival counter the host zeroes before the launches), then
    // reduces and updates its slice of the parameters with `adam`; CTA 0
    // advances adam.step.  NULL: partials only, k_mlp_adam follows.
    unsigned* grid_bar;
    AdamArgs adam;
};

// The view march (writes the samples, the step tables and sb.alpha).
cudaError_t launch_march(VolDesc vd, CamDesc cam, TraceParams tp, SampleBuf sb, bool hw,
                         cudaStream_t st);
cudaError_t launch_shade_exact(VolDesc vd, CamDesc cam, TraceParams tp, SampleBuf sb,
                               float4* out, cudaStream_t st);
cudaError_t launch_pack_level(VolDesc vd, int l, cudaSurfaceObject_t surf, cudaStream_t st);
cudaError_t launch_fbm_volume(TraceParams tp, const float org[3], const float ext[3], int R,
                              cudaSurfaceObject_t surf, cudaStream_t st);
// Surrogate shading on the tensor cores (k_shade_tc.cu).  status (4 words,
// zeroed before the launch): [0] += exact-cone fallbacks, [1] |= 1 when a
// bounded wait ran out, [2] += samples shaded, [3] tile claim counter.
cudaError_t launch_shade_mlp_tc(VolDesc vd, CamDesc cam, TraceParams tp, const MlpDev& m,
                                SampleBuf sb, unsigned long long* status, cudaStream_t st);
// One CTA waits on an mbarrier nothing arrives on, bounded by limit_ns
// (status: [1] |= 1 on the timeout, [3] = nanoseconds waited).
// The fused surrogate renderer (k_render_tc.cu): march, tensor-core MLP and
// composite in one persistent kernel.  contrib: per 8x4-pixel region
// (raster order, ceil(W/8) * ceil(H/4) of them) 32 * view_steps floats;
// steps: per region view_steps (first slot, lane ballot) pairs; dst: the
// finished image.  status (4 words, zeroed before the launch): [0] +=
// exact-cone fallbacks, [1] |= 1 when a bounded wait ran out (|= 2: and the
// drain after it), [2] += samples shaded, [3] region claim counter.
cudaError_t launch_render_mlp_tc(VolDesc vd, CamDesc cam, TraceParams tp, const MlpDev& m,
                                 float* contrib, uint2* steps, float4* dst,
                                 unsigned long long* status, cudaStream_t st);
cudaError_t launch_wait_probe(uint64_t limit_ns, unsigned long long* status, cudaStream_t st);
// dst: where the finished pixels go (a device image, or a device-addressable
// host image); their alpha comes from the march (sb.alpha)
cudaError_t launch_accumulate(CamDesc cam, TraceParams tp, SampleBuf sb, float4* dst,
                              cudaStream_t st);
cudaError_t launch_mlp_features(VolDesc vd, const MlpDev& m, const float* pos, int n,
                                const float dir[3], float* out, cudaStream_t st);
// network evaluation on the tensor cores (k_shade_tc.cu); status[1] |= 1 when
// a tensor-core wait ran out of its time limit
cudaError_t launch_mlp_infer(const MlpDev& m, const float* feat, int n, float* out,
                             unsigned long long* status, cudaStream_t st);
// one training step on the tensor cores (k_train_tc.cu); a tensor-core wait
// that ran out of its time limit sets ta.status and leaves a NaN in the CTA's
// loss slot
// One training step: partials only (ta.grid_bar NULL), or with the optimiser
// fused (cooperative launch; cudaErrorCooperativeLaunchTooLarge when ctas
// exceeds mlp_train_resident_ctas()).
cudaError_t launch_mlp_train(const TrainArgs& ta, int ctas, cudaStream_t st);
int mlp_train_resident_ctas();
cudaError_t launch_mlp_adam(const AdamArgs& aa, cudaStream_t st);

// Message returned by cg_last_error() on this thread (cg_host.cpp).
void set_last_error(const char* msg);

// Sun::update's frame for the box position + [b0, b1]^3 (FP32, fixed order;
// cg_host.cpp).  False when the sun is parallel to the up axis.
bool sun_frame_for_box(const float position[3], float b0, float b1, const float dir[3], int W,
                       int H, SunFrame& fr);

// ---- launchers (return cudaGetLastError of the launch) -------------------
cudaError_t launch_bin_count(const BoardsDev& b, int D, Bins bins, cudaStream_t st);
cudaError_t launch_bin_scan(Bins bins, cudaStream_t st);
cudaError_t launch_bin_fill(const BoardsDev& b, int D, Bins bins, cudaStream_t st);
cudaError_t launch_sunmap(const BoardsDev& b, const SunFrame& fr, uint64_t* keys,
                          cudaStream_t st);
// hl_brick (may be NULL): per 8^3 brick of the volume, set to 1 beside every
// mask byte set (cleared by the caller before the launch)
cudaError_t launch_highlight(const BoardsDev& b, const SunFrame& fr, const uint64_t* keys,
                             float4* posmap, int D, const float wmin[3],
                             const float range[3], float offset, uint8_t* mask,
                             uint8_t* hl_brick, cudaStream_t st);
// coverage_only: write the integer coverage (count, dq) and nothing else
cudaError_t launch_splat(const BoardsDev& b, Bins bins, const uint8_t* mask, VolDesc vd,
                         void* pyr, uint32_t* count, uint32_t* dq, int fused_levels,
                         OccRaw raw, bool coverage_only, cudaStream_t st);
cudaError_t launch_mip_level(VolDesc vd, void* pyr, int l, cudaStream_t st);
// levels l0+1 .. L-1 in one single-CTA launch (for levels of at most
// CG_MIP_TAIL_MAX parents each)
#define CG_MIP_TAIL_MAX 32768
cudaError_t launch_mip_tail(VolDesc vd, void* pyr, int l0, cudaStream_t st);
// Dilated occupancy grids of brick B = 1 << vd.occ_shift from the raw cells.
// Builds the brick grids from the raw cells and grows the level-0 occupied
// box (vd.occ_box, zeroed by the caller).
cudaError_t launch_occ_dilate(VolDesc vd, OccRaw raw, uint8_t* occ, int total, cudaStream_t st);
cudaError_t launch_count_active(const uint32_t* count, const uint8_t* mask, size_t n,
                                unsigned long long* out, cudaStream_t st);

cudaError_t launch_trace_fused(VolDesc vd, CamDesc cam, TraceParams tp, float4* out,
                               unsigned long long* stats, cudaStream_t st);
cudaError_t launch_noise_table(TraceParams tp, float* tab, int total, cudaStream_t st);
cudaError_t launch_trace_cones(VolDesc vd, TraceParams tp, const float* pos, int n,
                               float* out, cudaStream_t st);

// FP64 image error statistics (k_stats.cu): out[0..3] max |a - ref| per RGBA
// channel, out[4..7] sums of squared differences.
size_t err_stats_scratch_bytes();
cudaError_t launch_err_stats(const float4* a, const void* ref, int ref_f64, size_t n,
                             double* scratch, double* out, cudaStream_t st);

// Sun-cone schedule of a launch (k_trace.cu, host, FP64).
ConeSchedule make_cone_schedule(const VolDesc& vd, const TraceParams& tp);

// ---- batched rendering (k_batch.cu) -----------------------------------------
// One view of a batch: its volume, camera, parameters (sun and noise of its
// volume), cone schedule, output, and its tiles' numbers [tile0, tile0 +
// tiles_x * tiles_y).
struct BatchView {
    VolDesc vd;
    CamDesc cam;
    TraceParams tp;
    ConeSchedule cs;
    float4* out;
    int tiles_x, tiles_y;
    unsigned tile0;
    unsigned pad;
};
void batch_tiles(int lanes_per_ray, int width, int height, int& tiles_x, int& tiles_y);
cudaError_t launch_trace_batch(int fmt, int lanes_per_ray, int unroll, const BatchView* views,
                               int n, unsigned total_tiles, unsigned* counter, cudaStream_t st);


// ---- compat render (k_compat.cu) ------------------------------------------
// The reference's billboard image formation; see cg_render_compat.
constexpr int CG_COMPAT_TILE = 8;  // pixel tile edge
struct CompatDev {
    CamDesc cam;
    int n;                 // boards
    const float4* cwr;     // world centre, radius
    int tiles_x, tiles_y;
    float near_z;
    int show_quad, do_noise, do_cone;
    float step_size, noise_opacity;
    int octaves;
    float freq_step, pers_step, inv_adjust;
    int min_steps, max_steps;
    float min_color, color_scale;
    float off[3];
    float clear[4];
    float cutoff;
    float sun[3];
    const float2* noise;   // green and alpha of the decoded 32^3 noise map
};
// Per board: tile rectangle (x0, y0, x1, y1; empty when x0 > x1) and the
// squared eye distance; per tile: the number of boards whose quad may cover it;
// *pairs (64-bit) += every board's tile count.
cudaError_t launch_compat_count(const CompatDev& P, int4* rect, float* key, uint32_t* tile_count,
                                unsigned long long* pairs, cudaStream_t st);
// Per tile: (distance bits << 32 | board) at the tile's cursor.
cudaError_t launch_compat_fill(const CompatDev& P, const int4* rect, const float* key,
                               uint32_t* cursor, unsigned long long* list, cudaStream_t st);
// Per tile: order its list by distance and blend its pixels front to back.
cudaError_t launch_compat_tiles(const VolDesc& vd, const ConeSchedule& cs, const CompatDev& P,
                                const uint32_t* offset, unsigned long long* list, float4* out,
                                cudaStream_t st);
