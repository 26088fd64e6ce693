// cg_internal.h -- structures shared by the host library and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define CG_MAX_LEVELS 16
#define CG_Q20 1048576LL
#define CG_HALF_Q20 524288LL
#define CG_KEY_EMPTY 0xFFFFFFFFFFFFFFFFULL
#define CG_BRICK 8           // splat brick edge (voxels)
#define CG_FUSED_MIPS 3      // levels produced inside the splat kernel
#define CG_SPLAT_CHUNK 256   // boards staged in shared memory per pass

// Sun-view frame: lookAt basis + ortho window (Sun::update, Sun.hpp:26-43).
struct SunFrame {
    float eye[3], right[3], up[3], fwd[3], t[3];
    float lo, hi, near_z, clip;
    int W, H;
};

// Pyramid description passed by value to kernels.
//
// Occupancy: for every level l a grid of occ_nb[l]^3 bytes, one per brick of
// 8^3 level-l texels (level-0 bricks map to level-l bricks by b >> l).  A byte
// is 1 when the brick or one of its 26 neighbours holds a voxel with density
// R > 0.  Because the mips are means of non-negative values, a trilinear
// footprint whose brick reads 0 has R = 0 exactly, so samplers may skip it.
struct VolDesc {
    int D, L, fmt;
    int dims[CG_MAX_LEVELS];
    long long offs[CG_MAX_LEVELS];  // voxels
    float wmin[3], range[3];
    const void* pyr;                // float4* (RGBA32F) or uint32_t* (BF16_FP16)
    const uint8_t* occ;             // occupancy grids, concatenated by level
    int occ_nb[CG_MAX_LEVELS];
    int occ_off[CG_MAX_LEVELS];
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
    float tan_half, h0, rmin, lod_offset, down_scaling;
    float sigma, ambient, cutoff;
    float sun_color[3];
    float sun[3];   // unit direction toward the sun
    uint32_t noise_seed;
    int noise_octaves;
    float noise_freq, noise_lac, noise_gain, noise_inv_norm;
    NoiseTab nt;
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

struct Bins {
    int nbx, nby, nbz, nbricks;
    uint32_t* count;   // nbricks
    uint32_t* offset;  // nbricks + 1
    uint32_t* cursor;  // nbricks
    uint32_t* list;    // pairs
};

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
cudaError_t launch_highlight(const BoardsDev& b, const SunFrame& fr, const uint64_t* keys,
                             float4* posmap, int D, const float wmin[3],
                             const float range[3], float offset, uint8_t* mask,
                             cudaStream_t st);
cudaError_t launch_splat(const BoardsDev& b, Bins bins, const uint8_t* mask, VolDesc vd,
                         void* pyr, uint32_t* count, uint32_t* dq, int fused_levels,
                         uint8_t* occ, cudaStream_t st);
cudaError_t launch_mip_level(VolDesc vd, void* pyr, int l, cudaStream_t st);
cudaError_t launch_occ_dilate(VolDesc vd, const uint8_t* raw, uint8_t* occ, int total,
                              cudaStream_t st);
cudaError_t launch_count_active(const uint32_t* count, const uint8_t* mask, size_t n,
                                unsigned long long* out, cudaStream_t st);

cudaError_t launch_trace_fused(VolDesc vd, CamDesc cam, TraceParams tp, float4* out,
                               unsigned long long* stats, cudaStream_t st);
cudaError_t launch_noise_table(TraceParams tp, float* tab, int total, cudaStream_t st);
cudaError_t launch_trace_cones(VolDesc vd, TraceParams tp, const float* pos, int n,
                               float* out, cudaStream_t st);
