/*
 * cloudgb.h -- C ABI of the GB300-native volumetric cloud path.
 *
 * The path: spherical billboards -> sun-view nearest-surface map -> highlight
 * stores -> integer coverage/density volume -> 3D mip pyramid -> per-pixel
 * view march with a sun cone (exact, or an MLP surrogate).
 *
 * Every entry point replaces one piece of the reference's C++/GLSL surface
 * (jaafersheriff/Cloud-Renderer); the citation is given beside it.  The
 * reference had no FFI: its boundary was the OpenGL API (glBufferData,
 * glDrawArraysInstanced, glGenerateMipmap, glGetTexImage).  Here the boundary is
 * this header: plain pointers and sizes, opaque handles, status codes, no CUDA
 * or C++ types.  A `void* stream` argument is a cudaStream_t (NULL = the
 * context's own stream).
 *
 * Error behaviour: every call returns a cg_status and never aborts; the
 * message of the last failure on the calling thread is cg_last_error().
 * (Reference: GL errors were only printed, GLSL.hpp:40-44, and shader
 * failures called exit(), Shader.cpp:35-36.)
 *
 * Threading: a context and its volumes are used from one thread at a time.
 */
#ifndef CLOUDGB_H
#define CLOUDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLOUDGB_ABI_VERSION 2

typedef enum cg_status {
    CG_OK = 0,
    CG_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad enum, non-finite value */
    CG_ERR_OUT_OF_RANGE = 2,     /* size or value beyond a documented limit */
    CG_ERR_OUT_OF_MEMORY = 3,    /* device or host allocation failed */
    CG_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    CG_ERR_NOT_READY = 5,        /* call order: e.g. render before voxelize */
    CG_ERR_DEVICE_FAULT = 6,     /* a kernel raised its error flag */
    CG_ERR_IO = 7,               /* file open/read/write failed */
    CG_ERR_BAD_CHECKPOINT = 8,   /* wrong magic/version/shape/CRC */
    CG_ERR_UNSUPPORTED = 9       /* feature not available in this build */
} cg_status;

/* Volume storage format of the mip pyramid. */
typedef enum cg_format {
    CG_FORMAT_RGBA32F = 0,  /* 16 B/voxel: R density, G light, B count, A occupancy */
    CG_FORMAT_BF16_FP16 = 1 /* 4 B/voxel: bf16 density (low half), fp16 light (high half) */
} cg_format;

/* Sun-cone accumulation rule. */
typedef enum cg_cone_mode {
    CG_CONE_TRANSMITTANCE = 0, /* optical depth sum(R * dh), T = exp(-sigma tau) */
    CG_CONE_REFERENCE = 1      /* traceCone's sum(r * i / (steps*downScaling)) over the
                                  light channel, clamp-to-edge (conetrace_frag.glsl:64-79) */
} cg_cone_mode;

typedef struct cg_context cg_context;
typedef struct cg_volume cg_volume;
typedef struct cg_mlp cg_mlp;

/* Directional sun (reference: Sun::position + Sun::update, Sun.hpp:26-43).
 * direction points from the volume toward the sun.  The sun-view map is the
 * reference's position FBO (VoxelizeShader.cpp:136-167), window-sized there
 * (1280x720 by default, main.cpp:25-26). */
typedef struct cg_sun {
    float direction[3];
    int map_width;
    int map_height;
} cg_sun;

/* Pinhole camera (reference: Camera::getP/getV, Camera.cpp:59-60).
 * Image row 0 is the top row; RGBA32F output, row-major. */
typedef struct cg_camera {
    float eye[3];
    float target[3];
    float up[3];
    float fov_y_degrees;
    int width;
    int height;
} cg_camera;

/* Hash value-noise fBm that replaces the reference's 32^3 noise texture
 * (ConeTraceShader.cpp:127-159, noise3D conetrace_frag.glsl:103-120). */
typedef struct cg_noise {
    uint32_t seed;
    int octaves;      /* 0 = no noise (density not modulated) */
    float frequency;  /* base lattice frequency over world units */
    float lacunarity; /* reference freqStep */
    float gain;       /* reference persStep */
    /* Shift of the noise domain in base-frequency lattice units: octave k
     * samples noise_k((p * frequency + offset) * lacunarity^k).  The
     * reference's per-octave octaveOffsets = windVel * runTime
     * (ConeTraceShader.cpp:55-61), added to the noise coordinate before the
     * octave's frequency step (conetrace_frag.glsl:110); 0 = static noise. */
    float offset[3];
} cg_noise;

/* Render parameters (reference: ConeTraceShader public fields,
 * ConeTraceShader.hpp:15-32). */
typedef struct cg_render_params {
    int view_steps;            /* uniform view-march samples over the AABB chord */
    int sun_steps;             /* vctSteps */
    float cone_half_angle;     /* radians; the reference's vctConeAngle is 2x this */
    float cone_initial_height; /* vctConeInitialHeight, level-0 voxels */
    float cone_min_radius;     /* floor of the cone radius, level-0 voxels */
    float lod_offset;          /* vctLodOffset */
    float down_scaling;        /* vctDownScaling (CG_CONE_REFERENCE only) */
    float density_scale;       /* extinction sigma per unit density per world unit */
    float ambient;             /* light floor in [0,1] */
    float sun_color[3];
    float transmittance_cutoff;/* early ray termination threshold */
    int cone_mode;             /* cg_cone_mode */
    cg_noise noise;
    int use_mlp;               /* 1: sun cone replaced by the MLP surrogate */
    const cg_mlp* mlp;         /* required when use_mlp != 0 */
    int pipeline;              /* cg_pipeline */
    /* exact cone, fused pipeline: 0 = each thread traces the sun cones of
     * its own ray's samples; N in 1..32 = the warp marches its 32 rays in
     * lockstep and, at a view step where at most N of them contribute,
     * traces each of those cones with its lanes over the cone's steps (a
     * shuffle-tree sum; images within 1e-6 of N = 0).  Default 8 (the
     * fastest measured: 1080p over 256^3, 3 % faster than 0, while 32 is
     * six times slower) */
    int cone_lanes;
} cg_render_params;

/* Kernel organisation of an exact-cone render.  Both give the same image
 * (same samples, same per-pixel summation order). */
typedef enum cg_pipeline {
    /* exact cone: one thread per pixel marches and traces its cones;
     * MLP surrogate: the deferred form below (its fastest on GB300) */
    CG_PIPELINE_FUSED = 0,
    /* march records the contributing samples; the sun term is evaluated for
     * them in full warps (exact cone) or 128-row tensor-core tiles (MLP),
     * then each pixel sums its samples in step order */
    CG_PIPELINE_DEFERRED = 1,
    /* MLP surrogate only (CG_ERR_UNSUPPORTED for the exact cone): one
     * persistent warp-specialised kernel marches, runs the network on the
     * tensor cores and composites, with no sample records in global memory;
     * the same images as the deferred form, bit for bit, but slower on GB300
     * (the network's epilogue needs the warps the march takes).
     * view_steps <= 2047 (above, the deferred form) */
    CG_PIPELINE_PERSISTENT = 2
} cg_pipeline;

/* Snapshot of a volume's layout, for readback. */
typedef struct cg_volume_info {
    int dimension;
    int mips;
    int format;
    int board_count;
    float world_min[3];
    float world_max[3];
    int level_dim[16];
    size_t level_offset[16]; /* in voxels from the start of the pyramid */
    size_t bytes_per_voxel;
    size_t pyramid_bytes;
} cg_volume_info;

/* ---- library / context ------------------------------------------------- */

const char* cg_status_string(cg_status s);
/* Message of the last failing call on this thread ("" if none). */
const char* cg_last_error(void);
int cg_abi_version(void);

/* One context per device and host thread.  (Reference: the GL context made
 * by Window::init, Window.cpp:54-106.) */
cg_status cg_context_create(int device, cg_context** out);
void cg_context_destroy(cg_context* ctx);
cg_status cg_context_synchronize(cg_context* ctx);
/* Number of this library's kernels launched on the context so far. */
uint64_t cg_context_launch_count(const cg_context* ctx);
/* Fill p with the documented defaults. */
void cg_render_params_default(cg_render_params* p);
/* Per-stage CUDA-event timing (cf. the reference's FPS/dt counters,
 * Window.cpp:127-137): when on, cg_voxelize and cg_render record an event
 * after each stage; cg_context_stage_times returns the stage durations (ms)
 * of the last such call and their names, ';'-separated. */
cg_status cg_context_set_timing(cg_context* ctx, int enable);
cg_status cg_context_stage_times(cg_context* ctx, float* ms, int max_stages, int* count,
                                 char* names, size_t names_len);

/* Memory helpers so that callers without a CUDA binding can pass pinned host
 * or device buffers (the reference's VBO/texture storage, CloudVolume.cpp:27-48).
 * kind of cg_memcpy: 1 host->device, 2 device->host, 3 device->device. */
cg_status cg_host_alloc(size_t bytes, void** out);
void cg_host_free(void* p);
cg_status cg_device_alloc(size_t bytes, void** out);
void cg_device_free(void* p);
cg_status cg_memcpy(void* dst, const void* src, size_t bytes, int kind);

/* ---- CloudVolume ------------------------------------------------------- */

/* CloudVolume(int dim, vec2 bounds, vec3 position, int mips)
 * (CloudVolume.cpp:7-55).  World box = position + [bound_min, bound_max]^3.
 * mips <= floor(log2(dimension)) + 1; dimension in [2, 512]. */
cg_status cg_volume_create(cg_context* ctx, int dimension, float bound_min,
                           float bound_max, const float position[3], int mips,
                           int format, cg_volume** out);
void cg_volume_destroy(cg_volume* vol);

/* Billboard list upload (CloudVolume::uploadBillboards, CloudVolume.cpp:139-164,
 * with fluffiness multiplying the radii, :153-160).  positions: count*3 floats
 * relative to the volume position; scales: radii; densities: per-board density
 * (>= 0, < 32768; NULL = all 1).  Host pointers; copied before return. */
cg_status cg_volume_set_billboards(cg_volume* vol, const float* positions,
                                   const float* scales, const float* densities,
                                   int count, float fluffiness);
/* VoxelizeShader::voxelize(CloudVolume*) (VoxelizeShader.cpp:18-31): clear,
 * sun-view nearest-surface map (first_voxelize.glsl), highlight stores
 * (second_voxelize.glsl), coverage/density splat, and the mip pyramid
 * (glGenerateMipmap, VoxelizeShader.cpp:105). Asynchronous on stream. */
cg_status cg_voxelize(cg_volume* vol, const cg_sun* sun, void* stream);

/* ConeTraceShader::coneTrace(CloudVolume*) (ConeTraceShader.cpp:15-82):
 * per-pixel view march + sun cone.  rgba_out holds width*height*4 floats; it
 * is a host pointer (the call is synchronous) unless out_on_device.  Page-
 * locked host memory (cg_host_alloc) is written by the device as the pixels
 * are finished; other host memory receives one copy after the frame. */
cg_status cg_render(cg_context* ctx, const cg_volume* vol, const cg_camera* cam,
                    const cg_render_params* params, float* rgba_out,
                    int out_on_device, void* stream);

/* Render once with counting on (untimed measurement aid, cf. the reference's
 * Stats pane, main.cpp:144-155): counts[0] view samples evaluated, [1] sun
 * cones traced, [2] sun-cone samples taken, [3] pixels whose ray met the box. */
cg_status cg_render_stats(cg_context* ctx, const cg_volume* vol, const cg_camera* cam,
                          const cg_render_params* params, uint64_t counts[4]);

/* The march pass of the deferred renderer alone: every view sample that
 * contributes to the image (alpha > 0), as level-0 voxel positions (3 floats)
 * and compositing weights T*alpha, in pixel-tile order.  Writes at most
 * `capacity` samples; *count receives the total.  Used to draw training
 * samples for the surrogate from the renderer's own query distribution. */
cg_status cg_march_samples(cg_context* ctx, const cg_volume* vol, const cg_camera* cam,
                           const cg_render_params* params, float* positions, float* weights,
                           int capacity, int* count);

/* traceCone(sampler3D, position, direction, steps, angle, height)
 * (conetrace_frag.glsl:64-79) evaluated at n level-0 voxel-space positions
 * (n*3 floats) toward direction.  out[i] = optical depth (CG_CONE_TRANSMITTANCE)
 * or the reference's weighted sum (CG_CONE_REFERENCE).  Host pointers unless
 * on_device. */
cg_status cg_trace_cones(const cg_volume* vol, const float* positions, int n,
                         const float direction[3], const cg_render_params* params,
                         float* out, int on_device, void* stream);

/* ---- readback (reference: VoxelShader::updateVoxelData's glGetTexImage,
 * VoxelShader.cpp:102-133) -- synchronous, host destinations ------------- */

cg_status cg_volume_get_info(const cg_volume* vol, cg_volume_info* info);
/* Raw level contents in the volume's format (level_dim^3 voxels). */
cg_status cg_volume_read_level(const cg_volume* vol, int level, void* dst,
                               size_t dst_bytes);
/* Level-0 integer coverage of the last voxelize: per voxel board count and
 * Q16.16 density sum (computed on demand; CG_ERR_NOT_READY when the
 * billboards were replaced after that voxelize). */
cg_status cg_volume_read_coverage(const cg_volume* vol, uint32_t* count,
                                  uint32_t* density_q16);
/* Sun-view map of the last voxelize: keys (depth bits << 32 | board, or
 * ~0 = empty) and world positions (x, y, z, valid) per texel, row 0 = bottom. */
cg_status cg_volume_read_sun_map(const cg_volume* vol, uint64_t* keys,
                                 float* positions);
/* Level-0 highlight mask (second_voxelize.glsl stores), one byte per voxel. */
cg_status cg_volume_read_highlight(const cg_volume* vol, uint8_t* mask);
/* activeVoxels statistic (VoxelShader.cpp:110-119): voxels with count > 0 or
 * a highlight mark, counted on the device. */
cg_status cg_volume_active_voxels(const cg_volume* vol, uint64_t* active);

/* ---- MLP sun-transmittance surrogate ------------------------------------
 * No counterpart in the reference (its traceCone is the exact method).  A
 * SiLU network of 3 (default), 2 or 1 hidden layers of width 64 (16 -> 64
 * [-> 64 [-> 64]] -> 1) predicts the sun cone's optical depth from 16
 * features of a view sample:
 *   f[3i+k] = density at level base_level+i sampled at
 *             v + (initial_height + (k + 0.5) * 2^(base_level+i)) * s  (i<4, k<3)
 *   f[12..14] = v / dimension,  f[15] = s.y
 * (v: level-0 voxel position, s: unit sun direction).  FP16 weights and
 * activations on the tensor cores, FP32 accumulation and master weights.
 * Training, inference and the render use the project's own kernels.  The
 * parameter vector always has the three-layer layout (CG_MLP_PARAMS floats);
 * a shallower model keeps the blocks of the layers it does not use at zero. */
#define CG_MLP_FEATURES 16
#define CG_MLP_PARAMS 9473
#define CG_MLP_MAX_LAYERS 3
#define CG_MLP_DEFAULT_LAYERS 3

typedef struct cg_mlp_config {
    int base_level;        /* feature levels base_level .. base_level+3 */
    float initial_height;  /* feature offsets start here (level-0 voxels) */
    /* the volume resolution and exact cone the model replaces; cg_render
     * rejects a model whose values differ from the render's */
    int dimension;
    int sun_steps;
    float cone_half_angle, cone_initial_height, cone_min_radius, lod_offset;
    /* input normalisation x = (f - mean) / stddev, output tau = tau_scale * softplus(y) */
    float mean[CG_MLP_FEATURES], stddev[CG_MLP_FEATURES];
    /* trusted feature range: samples outside use the exact cone */
    float feature_min[CG_MLP_FEATURES], feature_max[CG_MLP_FEATURES];
    float tau_scale;
} cg_mlp_config;

typedef struct cg_train_params {
    int steps;        /* optimiser steps */
    int batch;        /* rows per step, multiple of 128 */
    float lr, beta1, beta2, eps; /* Adam */
    float sigma;      /* extinction of the loss (exp(-sigma tau_pred) - exp(-sigma tau))^2 */
    uint64_t seed;    /* batch permutation */
    int separate_adam; /* 0 (default): Adam runs inside the training launch when the
                          batch's CTAs fit on the GPU at once (batch <= 128 x the
                          resident CTAs, 19456 rows on 152 SMs), else as a second
                          launch; 1: always the second launch.  Same results. */
} cg_train_params;

void cg_mlp_config_default(cg_mlp_config* c);
void cg_train_params_default(cg_train_params* p);
int cg_mlp_param_count(void);
/* He-uniform initialisation from a SplitMix64 stream seeded with `seed`;
 * CG_MLP_DEFAULT_LAYERS hidden layers. */
cg_status cg_mlp_create(cg_context* ctx, uint64_t seed, cg_mlp** out);
/* The same with 1 .. CG_MLP_MAX_LAYERS hidden layers (fixed for the model's
 * life; checkpoints record it).  Two layers shade ~25 % faster at the same
 * held-out accuracy on the 1080p workload. */
cg_status cg_mlp_create_layers(cg_context* ctx, uint64_t seed, int hidden_layers, cg_mlp** out);
int cg_mlp_hidden_layers(const cg_mlp* mlp);
void cg_mlp_destroy(cg_mlp* mlp);
cg_status cg_mlp_configure(cg_mlp* mlp, const cg_mlp_config* config);
cg_status cg_mlp_get_config(const cg_mlp* mlp, cg_mlp_config* config);
/* Raw features (n*16) at n level-0 voxel positions (n*3) of a voxelized volume. */
cg_status cg_mlp_features(const cg_volume* vol, const cg_mlp* mlp, const float* positions, int n,
                          const float direction[3], float* out, int on_device, void* stream);
/* Optical depth predicted from raw features (n*16 -> n). */
cg_status cg_mlp_infer(const cg_mlp* mlp, const float* features, int n, float* out,
                       int on_device, void* stream);
/* Mean loss and its gradient (CG_MLP_PARAMS floats, host) over n rows,
 * without an update: the training step's forward and backward kernels
 * (CG_ERR_DEVICE_FAULT when one of their bounded waits ran out). */
cg_status cg_mlp_gradient(cg_mlp* mlp, const float* features, const float* tau, int n,
                          float sigma, float* grad, float* loss, int on_device);
/* Train on n device-resident rows (features n*16, exact optical depth n).
 * Every tensor-core wait of the training kernel is bounded (1 s): when one
 * runs out, no update is made from that step on (parameters, Adam moments and
 * step stay as the last completed step left them), the remaining entries of
 * loss_per_step are NaN and the call returns CG_ERR_DEVICE_FAULT. */
cg_status cg_mlp_train(cg_mlp* mlp, const float* d_features, const float* d_tau, long long n,
                       const cg_train_params* params, float* loss_per_step);
/* Failure-detection check of the training kernels (no reference counterpart):
 * `steps` (1 .. 50) training steps of 1024 rows over n device-resident rows in
 * which the tensor-core layer barrier is never completed (no MMA is issued),
 * with every bounded wait limited to limit_us (1 .. 1e6).  The waits must run
 * out: returns CG_ERR_DEVICE_FAULT with no update made (parameters, Adam
 * moments and step unchanged), and the context stays usable.  CG_OK would
 * mean the bound did not fire. */
cg_status cg_mlp_check_train_timeout(cg_mlp* mlp, const float* d_features, const float* d_tau,
                                     long long n, int steps, uint32_t limit_us);
/* FP32 parameters (W stored [out][in]: W1 16x64, b1, W2, b2, W3, b3, W4, b4),
 * Adam moments and step; m, v, step may be NULL. */
cg_status cg_mlp_get_params(const cg_mlp* mlp, float* params, float* adam_m, float* adam_v,
                            int* step);
cg_status cg_mlp_set_params(cg_mlp* mlp, const float* params, const float* adam_m,
                            const float* adam_v, int step);
/* Versioned checkpoint (magic, version, shapes, config, params, Adam state,
 * step, CRC32); training resumes bit-identically from it. */
cg_status cg_mlp_save(const cg_mlp* mlp, const char* path);
cg_status cg_mlp_load(cg_context* ctx, const char* path, cg_mlp** out);
/* No counterpart in the reference.  Error statistics of an RGBA32F image
 * against a reference image (RGBA, FP64 when reference_is_f64, else FP32),
 * reduced on the GPU in FP64 with a fixed reduction order: out[0..3] max-abs
 * per channel, out[4..7] RMSE per channel, out[8] max-abs over all channels,
 * out[9] RMSE over all channels.  Host pointers unless on_device.  Blocks
 * until the result is on the host. */
cg_status cg_image_error_stats(cg_context* ctx, const float* image, const void* reference,
                               int reference_is_f64, uint64_t pixels, int on_device,
                               double out[10], void* stream);
/* Samples of the last MLP render that fell back to the exact cone.  Returns
 * CG_ERR_DEVICE_FAULT when that render's tensor-core pass stopped on a bounded
 * wait (the image is then incomplete). */
cg_status cg_context_mlp_fallbacks(cg_context* ctx, uint64_t* out);
/* View samples the last MLP render shaded (one surrogate inference each). */
cg_status cg_context_last_samples(cg_context* ctx, uint64_t* samples);
/* Failure-detection check (no reference counterpart): one CTA waits on a
 * tensor-core mbarrier that nothing completes, with the same bounded wait the
 * surrogate kernel uses, limited to limit_us (1 .. 1e6).  The wait must run
 * out: returns CG_ERR_DEVICE_FAULT with *waited_us = the time waited, and the
 * context stays usable.  CG_OK would mean the bound did not fire. */
cg_status cg_context_check_wait_timeout(cg_context* ctx, uint32_t limit_us, uint64_t* waited_us);

/* Bounds-check build (no reference counterpart; the stand-in for a memory
 * checker): cg_bounds_check_build() is 1 when the library was built with
 * CG_BOUNDS_CHECK=1, whose kernels test their global gather and scatter
 * indexes, skip an out-of-range access and count it instead of faulting.
 * cg_context_bounds_violations returns the count since its last call
 * (clearing it) and, in site (may be NULL), the first one's source line and
 * index; CG_ERR_UNSUPPORTED in the normal build.  Synchronises the device. */
int cg_bounds_check_build(void);
cg_status cg_context_bounds_violations(cg_context* ctx, uint64_t* count, char* site,
                                       int site_len);

/* ---- allocation-free variant ------------------------------------------- */

/* No counterpart in the reference.  The sun-view nearest-surface map and its
 * highlight stores (the first two passes of cg_voxelize) for callers that
 * cannot allocate device memory: hosts that own all device memory through
 * their own fixed budget, and real-time threads that cannot take cudaMalloc's
 * implicit synchronisation.  The call allocates nothing.  The caller passes
 * d_boards (count * 4 floats in device memory: world-space centre xyz =
 * volume position + board position, and radius = scale * fluffiness) and
 * the two outputs in device memory: d_positions (map_width * map_height * 4
 * floats, cg_volume_read_sun_map's layout) and d_mask (dimension^3 bytes,
 * cleared by the call, cg_volume_read_highlight's layout).  The per-texel depth
 * keys live in a fixed array inside the library of CG_NOALLOC_MAX_TEXELS keys
 * (8 MiB), held by every GPU that loads the library until the process exits;
 * larger sun maps are rejected with CG_ERR_OUT_OF_RANGE.  The first call on a
 * device looks up that array's device address (make it before any stream
 * capture).  All calls share the array: calls that overlap on the GPU race,
 * so serialise them.  Asynchronous on stream (NULL = the legacy default
 * stream); results match cg_voxelize's sun map and highlight mask bit for bit. */
#define CG_NOALLOC_MAX_TEXELS (1 << 20)
cg_status cg_sun_map_noalloc(int dimension, float bound_min, float bound_max,
                             const float position[3], const float* d_boards, int count,
                             const cg_sun* sun, float* d_positions, uint8_t* d_mask,
                             void* stream);

/* ---- many volumes and views per frame --------------------------------------
 * No counterpart in the reference (it renders one volume for one camera per
 * frame).  These serve the batching workload: many independent clouds and
 * views of uneven sizes rendered in one persistent launch, a whole frame
 * (every voxelize plus the batch render) replayed as one CUDA graph, and an
 * autotuner for the launch shape. */

/* Occupancy brick edge (4, 8 or 16 texels) of a volume's empty-space grids;
 * rendered images do not depend on it (empty bricks read exactly 0). */
cg_status cg_volume_set_occupancy_brick(cg_volume* vol, int brick);

/* Launch shape of the fused renderer: lanes per ray 1 (one ray per thread,
 * 32 rays per warp), 4, 8 or 32 (one ray per warp); step-loop unroll 1, 2 or 4;
 * occupancy brick 4, 8 or 16 (0 = leave the volumes' own). */
typedef struct cg_trace_config {
    int lanes_per_ray;
    int step_unroll;
    int brick;
} cg_trace_config;

/* One view of a batch: a voxelized volume of the context, a camera, and a
 * device buffer of width * height RGBA32F pixels (row 0 = top). */
typedef struct cg_batch_view {
    const cg_volume* volume;
    cg_camera camera;
    float* rgba_out;
} cg_batch_view;

/* Render n views with the plain FP32 exact method (params->use_mlp = 0,
 * fused pipeline) in one persistent launch; config NULL = the context's
 * (cg_context_set_trace_config / cg_autotune).  Images equal cg_render's for
 * every configuration.  The launch is asynchronous on `stream`; the call
 * first waits for the context's previous batch upload. */
cg_status cg_render_batch(cg_context* ctx, const cg_batch_view* views, int n,
                          const cg_render_params* params, const cg_trace_config* config,
                          void* stream);
cg_status cg_context_set_trace_config(cg_context* ctx, const cg_trace_config* config);
cg_status cg_context_get_trace_config(const cg_context* ctx, cg_trace_config* config);

/* Time every configuration (lanes per ray x unroll x brick, 36 of them) on a
 * batch, keep the fastest as the context's and apply its brick to the
 * volumes.  ms (optional, 36 entries) receives each configuration's time in
 * the order lanes (1, 4, 8, 32) x unroll (1, 2, 4) x brick (4, 8, 16), brick
 * fastest.  Blocks. */
cg_status cg_autotune(cg_context* ctx, const cg_batch_view* views, int n,
                      const cg_render_params* params, int repeats, cg_trace_config* best,
                      float* ms);

/* A frame as one CUDA graph: voxelize each volume with `sun`, then the batch
 * render, captured once (after one eager run that allocates) and replayed by
 * cg_frame_graph_launch.  The volumes, views and parameters are fixed at
 * creation; billboards may be re-uploaded between launches with the same
 * count (cg_volume_set_billboards). */
typedef struct cg_frame_graph cg_frame_graph;
cg_status cg_frame_graph_create(cg_context* ctx, cg_volume* const* volumes, int nvol,
                                const cg_sun* sun, const cg_batch_view* views, int nviews,
                                const cg_render_params* params, cg_frame_graph** out);
cg_status cg_frame_graph_launch(cg_frame_graph* graph, void* stream);
void cg_frame_graph_destroy(cg_frame_graph* graph);

/* ---- compat render: the reference's own image formation ------------------
 * ConeTraceShader::coneTrace (ConeTraceShader.cpp:15-82) as the reference
 * draws it: one camera-facing billboard of radius scale * fluffiness per
 * board (billboard_vert_instanced.glsl), shaded by the fragment program of
 * conetrace_frag.glsl:122-201 (soft-particle noise march through the board's
 * sphere, traceCone from the sphere surface toward the sun over the light
 * channel), blended SRC_ALPHA / ONE_MINUS_SRC_ALPHA over the clear colour in
 * distance order (main.cpp:94-95, sortBoards CloudVolume.cpp:65-82), without
 * a global sort: boards are binned to 8x8-pixel tiles and each tile orders
 * its own list.  Field names follow ConeTraceShader.hpp:15-32. */
typedef struct cg_compat_params {
    int show_quad;              /* showQuad: debug quad (sphere profile, white border) */
    int do_noise;               /* doNoiseSample */
    int do_cone_trace;          /* doConeTrace */
    float step_size;            /* stepSize, noise-map units */
    float noise_opacity;        /* noiseOpacity */
    int num_octaves;            /* numOctaves */
    float freq_step;            /* freqStep */
    float pers_step;            /* persStep */
    float adjust_size;          /* adjustSize: world units per noise-map period */
    int min_noise_steps;        /* minNoiseSteps (>= 2) */
    int max_noise_steps;        /* maxNoiseSteps (>= minNoiseSteps) */
    float min_noise_color;      /* minNoiseColor */
    float noise_color_scale;    /* noiseColorScale */
    float octave_offsets[3];    /* windVel * runTime (ConeTraceShader.cpp:55-61); octave k
                                   adds component k (k < 3) to all three coordinates */
    uint32_t noise_seed;        /* seed of the 32^3 noise map (initNoiseMap) */
    int vct_steps;              /* vctSteps (<= 64) */
    float vct_cone_angle;       /* vctConeAngle (full aperture, radians) */
    float vct_cone_initial_height; /* vctConeInitialHeight, level-0 voxels */
    float vct_lod_offset;       /* vctLodOffset */
    float vct_down_scaling;     /* vctDownScaling */
    float clear_color[4];       /* glClearColor (main.cpp:112) */
    float near_plane;           /* camera near plane (Camera.cpp:59); far = 2500 */
    float transmittance_cutoff; /* stop a pixel once the boards in front leave less than
                                   this of the background visible (0 = blend every board) */
} cg_compat_params;

/* The reference's defaults (ConeTraceShader.hpp:15-32, main.cpp:112). */
void cg_compat_params_default(cg_compat_params* p);

/* The decoded 32^3 RGBA noise map of a seed (initNoiseMap,
 * ConeTraceShader.cpp:127-159, from a seeded stream; exact integer
 * arithmetic): 32*32*32*4 floats, x fastest.  Host only, no device needed. */
cg_status cg_compat_noise_map(uint32_t seed, float* out);

/* Render the compat image of the volume's billboards.  The volume must have
 * been voxelized when do_cone_trace is set (the cone reads its light
 * channel; the sun is the one of that voxelize).  rgba_out as in cg_render
 * (row 0 = top); one host synchronisation sizes the tile lists. */
cg_status cg_render_compat(cg_context* ctx, const cg_volume* vol, const cg_camera* cam,
                           const cg_compat_params* params, float* rgba_out, int out_on_device,
                           void* stream);

#ifdef __cplusplus
}
#endif

#endif /* CLOUDGB_H */
