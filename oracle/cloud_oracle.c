/*
 * cloud_oracle.c -- CPU restatement of the reference's volumetric cloud path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke entry
 * and the bench's CPU-baseline leg load it; the product library never does.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures, and
 * its GL path cannot run without a graphics stack.  The restatement is pinned
 * against the reference's own shader functions compiled as C++ through a GLSL
 * shim (oracle/ref_shim/, built by oracle/build_ref.py into oracle/_ref/), which
 * generated the fixtures in tests/golden/.  Parts the reference has no code
 * for (the paper's sphere fill, the transmittance cone, the view march, the
 * hash noise, the MLP) are build-defined and pinned only by known-answer tests.
 *
 * Two builds of this one source:
 *   -DOR_REAL=double -> oracle/liboracle64.so, the FP64 oracle;
 *   -DOR_REAL=float  -> oracle/liboracle32.so, the FP32 multithreaded CPU baseline.
 * Index-deciding arithmetic (sun-view depth keys, highlight voxel indices) is
 * FP32 in both builds with a fixed operation order; build with
 * -ffp-contract=off so that no FMA is formed.  Coverage is integer (Q20 fixed
 * point) and identical in both builds.
 *
 * Reference citations are paths inside jaafersheriff/Cloud-Renderer.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef OR_REAL
#define OR_REAL double
#endif
typedef OR_REAL real;

#define OR_API __attribute__((visibility("default")))
#define Q20 1048576LL
#define HALF_Q20 524288LL
#define KEY_EMPTY 0xFFFFFFFFFFFFFFFFULL

/* ------------------------------------------------------------------ */
/* parallel for                                                        */
/* ------------------------------------------------------------------ */
typedef void (*or_task_fn)(void* ctx, long i);
typedef struct {
    or_task_fn fn;
    void* ctx;
    long n;
    atomic_long next;
} or_pool_job;

static void* or_worker(void* arg) {
    or_pool_job* job = (or_pool_job*)arg;
    for (;;) {
        long i = atomic_fetch_add(&job->next, 1);
        if (i >= job->n) break;
        job->fn(job->ctx, i);
    }
    return NULL;
}

static void or_parallel_for(long n, int nthreads, or_task_fn fn, void* ctx) {
    or_pool_job job;
    job.fn = fn;
    job.ctx = ctx;
    job.n = n;
    atomic_init(&job.next, 0);
    if (nthreads <= 1 || n <= 1) {
        or_worker(&job);
        return;
    }
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    int started = 0;
    for (int t = 0; t < nthreads - 1; ++t)
        if (pthread_create(&th[t], NULL, or_worker, &job) == 0) started++;
        else break;
    or_worker(&job);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* FP32 vector helpers (fixed order; -ffp-contract=off)                 */
/* ------------------------------------------------------------------ */
typedef struct { float x, y, z; } f3;

static f3 f3_make(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static f3 f3_sub(f3 a, f3 b) { return f3_make(a.x - b.x, a.y - b.y, a.z - b.z); }
static float f3_dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
/* cross(x, y) in GLM's component order */
static f3 f3_cross(f3 a, f3 b) {
    return f3_make(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
/* normalize(v) = v * inversesqrt(dot(v, v)), inversesqrt = 1/sqrt */
static f3 f3_normalize(f3 v) {
    float inv = 1.0f / sqrtf(f3_dot(v, v));
    return f3_make(v.x * inv, v.y * inv, v.z * inv);
}

/* ------------------------------------------------------------------ */
/* Sun frame: Sun::update (Sun.hpp:26-43) with a directional sun.        */
/* ------------------------------------------------------------------ */
typedef struct {
    float eye[3];   /* lookPos */
    float right[3]; /* s of lookAt */
    float up[3];    /* u of lookAt */
    float fwd[3];   /* f of lookAt (= lookDir) */
    float t[3];     /* view translation: -dot(s,eye), -dot(u,eye), dot(f,eye) */
    float lo, hi;   /* ortho window [lo,hi]^2 (minmin, maxmax) */
    float near_z;   /* near distance 0.01 */
    float clip;     /* clipDistance */
    int W, H;
} or_sun_frame;

/* Returns 0 on success, -1 when the sun is parallel to the up axis. */
OR_API int or_sun_frame_make(const float position[3], float b0, float b1,
                             const float dir[3], int W, int H, or_sun_frame* fr) {
    f3 pos = f3_make(position[0], position[1], position[2]);
    f3 s = f3_make(dir[0], dir[1], dir[2]);
    /* lookDir = normalize(vol->position - Sun::position) (Sun.hpp:30); the sun
     * at infinity along s gives -s. */
    f3 lookDir = f3_normalize(f3_make(-s.x, -s.y, -s.z));
    f3 mn = f3_make(b0, b0, b0), mx = f3_make(b1, b1, b1);
    float minLen = sqrtf(f3_dot(mn, mn)), maxLen = sqrtf(f3_dot(mx, mx));
    float dist = minLen > maxLen ? minLen : maxLen;
    f3 lookPos = f3_make(pos.x - lookDir.x * dist, pos.y - lookDir.y * dist,
                         pos.z - lookDir.z * dist);
    /* glm::lookAt(lookPos, position, (0,1,0)) */
    f3 f = f3_normalize(f3_sub(pos, lookPos));
    f3 upv = f3_make(0.0f, 1.0f, 0.0f);
    f3 c = f3_cross(f, upv);
    float cl = f3_dot(c, c);
    if (!(cl > 1e-12f)) return -1;
    f3 r = f3_normalize(c);
    f3 u = f3_cross(r, f);
    fr->eye[0] = lookPos.x; fr->eye[1] = lookPos.y; fr->eye[2] = lookPos.z;
    fr->right[0] = r.x; fr->right[1] = r.y; fr->right[2] = r.z;
    fr->up[0] = u.x; fr->up[1] = u.y; fr->up[2] = u.z;
    fr->fwd[0] = f.x; fr->fwd[1] = f.y; fr->fwd[2] = f.z;
    fr->t[0] = -f3_dot(r, lookPos);
    fr->t[1] = -f3_dot(u, lookPos);
    fr->t[2] = f3_dot(f, lookPos);
    /* minmin/maxmax (Sun.hpp:34-35), ortho box (Sun.hpp:42) */
    fr->lo = 2.0f * b0;
    fr->hi = 2.0f * b1;
    fr->near_z = 0.01f;
    /* nearPlane/farPlane/clipDistance (Sun.hpp:37-40) */
    f3 np = f3_make(lookPos.x + lookDir.x * 0.01f, lookPos.y + lookDir.y * 0.01f,
                    lookPos.z + lookDir.z * 0.01f);
    float two_d = 2.0f * dist;
    f3 fp = f3_make(lookPos.x + lookDir.x * two_d, lookPos.y + lookDir.y * two_d,
                    lookPos.z + lookDir.z * two_d);
    f3 dd = f3_sub(np, fp);
    fr->clip = sqrtf(f3_dot(dd, dd));
    fr->W = W;
    fr->H = H;
    return 0;
}

/* Board centre in sun view space: V * (cw, 1) with the lookAt rows. */
static f3 sun_view_of(const or_sun_frame* fr, f3 cw) {
    f3 r = f3_make(fr->right[0], fr->right[1], fr->right[2]);
    f3 u = f3_make(fr->up[0], fr->up[1], fr->up[2]);
    f3 f = f3_make(fr->fwd[0], fr->fwd[1], fr->fwd[2]);
    f3 nf = f3_make(-f.x, -f.y, -f.z);
    return f3_make(f3_dot(r, cw) + fr->t[0], f3_dot(u, cw) + fr->t[1],
                   f3_dot(nf, cw) + fr->t[2]);
}

/* Texel centre of the ortho sun view (window pixel centre i+0.5). */
static float texel_x(const or_sun_frame* fr, int i) {
    float a = (float)i + 0.5f;
    float b = a / (float)fr->W;
    return fr->lo + b * (fr->hi - fr->lo);
}
static float texel_y(const or_sun_frame* fr, int j) {
    float a = (float)j + 0.5f;
    float b = a / (float)fr->H;
    return fr->lo + b * (fr->hi - fr->lo);
}

/* first_voxelize.glsl:40-63 for one fragment of one board, restated
 * analytically in sun view space.  The billboard faces the sun
 * (billboard_vert_instanced.glsl:20-38): its fragment at texel (xv, yv) lies in
 * the plane z = cv.z; the spherical profile is sqrt(max(0, 1-(d/r)^2)) with a
 * discard below 0.01 (first_voxelize.glsl:43-48); the surface point is pushed
 * toward the sun by r*profile (:52,:61); depth is the distance from the
 * near-plane point (0,0,-near) (:63).  Returns 1 when covered. */
static int sun_fragment(float xv, float yv, f3 cv, float r, float near_z,
                        float* zs_out, float* depth_out) {
    float dx = xv - cv.x;
    float dy = yv - cv.y;
    float d2 = dx * dx + dy * dy;
    float dist = sqrtf(d2);
    float q = dist / r;
    float t = 1.0f - q * q;
    float prof = sqrtf(t > 0.0f ? t : 0.0f);
    if (!(prof >= 0.01f)) return 0;
    float zs = cv.z + r * prof;
    float dz = zs + near_z;
    float dep2 = (xv * xv + yv * yv) + dz * dz;
    *zs_out = zs;
    *depth_out = sqrtf(dep2);
    return 1;
}

static uint32_t f32_bits(float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    return u;
}

/* ------------------------------------------------------------------ */
/* Volume                                                              */
/* ------------------------------------------------------------------ */
typedef struct {
    int D, L;
    float pos[3], b0, b1;
    float wmin[3], wmax[3], range[3];
    int dims[16];
    size_t offs[16];
    size_t total;
    real* rgba; /* pyramid, 4 channels per voxel */
    uint32_t* count;
    uint32_t* dq;
    uint8_t* mask;
    uint64_t* keys;
    float* posmap;
    int mapW, mapH;
    or_sun_frame frame;
    /* boards */
    int n;
    float* cw;  /* world centres, 3 per board */
    float* rad; /* radii = scale * fluffiness */
    int64_t* q; /* Q20 voxel-space centres, 3 per board */
    int64_t* rq;
    uint64_t* thr;
    uint32_t* dqb;
    uint8_t* culled;
} or_volume;

OR_API or_volume* or_volume_new(int D, float b0, float b1, const float pos[3], int L) {
    if (D < 2 || L < 1 || L > 16) return NULL;
    or_volume* v = (or_volume*)calloc(1, sizeof(or_volume));
    v->D = D;
    v->L = L;
    v->b0 = b0;
    v->b1 = b1;
    for (int a = 0; a < 3; ++a) {
        v->pos[a] = pos[a];
        /* world bounds = position + bounds (VoxelizeShader.cpp:124-126) */
        v->wmin[a] = pos[a] + b0;
        v->wmax[a] = pos[a] + b1;
        /* range = bounds.y - bounds.x, computed from the world bounds as in
         * calculateVoxelLerp (first_voxelize.glsl:24-26) */
        v->range[a] = v->wmax[a] - v->wmin[a];
    }
    size_t off = 0;
    for (int l = 0; l < L; ++l) {
        int n = D >> l;
        if (n < 1) n = 1;
        v->dims[l] = n;
        v->offs[l] = off;
        off += (size_t)n * n * n;
    }
    v->total = off;
    size_t n0 = (size_t)D * D * D;
    v->rgba = (real*)calloc(off * 4, sizeof(real));
    v->count = (uint32_t*)calloc(n0, 4);
    v->dq = (uint32_t*)calloc(n0, 4);
    v->mask = (uint8_t*)calloc(n0, 1);
    return v;
}

static void free_boards(or_volume* v) {
    free(v->cw); free(v->rad); free(v->q); free(v->rq); free(v->thr);
    free(v->dqb); free(v->culled);
    v->cw = v->rad = NULL; v->q = v->rq = NULL; v->thr = NULL; v->dqb = NULL;
    v->culled = NULL;
    v->n = 0;
}

OR_API void or_volume_free(or_volume* v) {
    if (!v) return;
    free(v->rgba); free(v->count); free(v->dq); free(v->mask);
    free(v->keys); free(v->posmap);
    free_boards(v);
    free(v);
}

OR_API int or_volume_total(const or_volume* v) { return (int)v->total; }
OR_API long or_volume_level_offset(const or_volume* v, int l) { return (long)v->offs[l]; }
OR_API int or_volume_level_dim(const or_volume* v, int l) { return v->dims[l]; }

static int64_t floor_div(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

/* Voxel bbox of a board along one axis: voxels whose centre (2i+1)*2^19 lies
 * within [q - rq, q + rq], clamped to [0, D-1].  Returns 0 if empty. */
static int board_axis_range(int64_t q, int64_t rq, int D, int* lo, int* hi) {
    int64_t l = floor_div(q - rq - HALF_Q20 + Q20 - 1, Q20);
    int64_t h = floor_div(q + rq - HALF_Q20, Q20);
    if (l < 0) l = 0;
    if (h > D - 1) h = D - 1;
    if (l > h) return 0;
    *lo = (int)l;
    *hi = (int)h;
    return 1;
}

/* Board list (CloudVolume::uploadBillboards, CloudVolume.cpp:139-164):
 * world centre = volumePosition + boardPosition (billboard_vert_instanced.glsl:21),
 * radius = scale * fluffiness.  Quantization to the Q20 voxel grid (FP64,
 * round-to-nearest-even):
 *   v  = (cw - wmin) / range * D            per axis
 *   q  = rint(v * 2^20)                     (board culled from coverage when v
 *                                            is outside [-D, 2D])
 *   rq = rint(r / range_x * D * 2^20)       (error when r > range_x)
 *   thr = floor(rq^2 * 9999 / 10000)        (profile >= 0.01 <=> d^2 <= 0.9999 r^2)
 *   dq = rint(density * 2^16)               (Q16.16)
 * Returns 0, or -1 (invalid) / -2 (out of range). */
OR_API int or_volume_set_boards(or_volume* v, const float* positions, const float* scales,
                                const float* dens, int n, float fluff) {
    free_boards(v);
    if (n < 0) return -1;
    v->n = n;
    size_t nn = n > 0 ? (size_t)n : 1;
    v->cw = (float*)malloc(nn * 3 * 4);
    v->rad = (float*)malloc(nn * 4);
    v->q = (int64_t*)malloc(nn * 3 * 8);
    v->rq = (int64_t*)malloc(nn * 8);
    v->thr = (uint64_t*)malloc(nn * 8);
    v->dqb = (uint32_t*)malloc(nn * 4);
    v->culled = (uint8_t*)malloc(nn);
    for (int b = 0; b < n; ++b) {
        float r = scales[b] * fluff;
        float d = dens ? dens[b] : 1.0f;
        if (!isfinite(r) || r < 0.0f || !isfinite(d) || d < 0.0f || d >= 32768.0f) return -1;
        int cull = 0;
        for (int a = 0; a < 3; ++a) {
            float c = v->pos[a] + positions[3 * b + a];
            if (!isfinite(c)) return -1;
            v->cw[3 * b + a] = c;
            double vv = ((double)c - (double)v->wmin[a]) / (double)v->range[a] * (double)v->D;
            if (!(vv >= -(double)v->D && vv <= 2.0 * (double)v->D)) {
                cull = 1;
                v->q[3 * b + a] = 0;
            } else {
                v->q[3 * b + a] = llrint(vv * (double)Q20);
            }
        }
        v->rad[b] = r;
        double rv = (double)r / (double)v->range[0] * (double)v->D;
        if (rv > (double)v->D) return -2;
        int64_t rq = llrint(rv * (double)Q20);
        v->rq[b] = rq;
        unsigned __int128 r2 = (unsigned __int128)(uint64_t)rq * (uint64_t)rq;
        v->thr[b] = (uint64_t)((r2 * 9999u) / 10000u);
        v->dqb[b] = (uint32_t)llrint((double)d * 65536.0);
        if (!cull) {
            int lo, hi;
            for (int a = 0; a < 3; ++a)
                if (!board_axis_range(v->q[3 * b + a], rq, v->D, &lo, &hi)) cull = 1;
        }
        v->culled[b] = (uint8_t)cull;
    }
    return 0;
}

OR_API void or_volume_get_quantized(const or_volume* v, int64_t* q, int64_t* rq,
                                    uint64_t* thr, uint32_t* dq, uint8_t* culled) {
    memcpy(q, v->q, (size_t)v->n * 3 * 8);
    memcpy(rq, v->rq, (size_t)v->n * 8);
    memcpy(thr, v->thr, (size_t)v->n * 8);
    memcpy(dq, v->dqb, (size_t)v->n * 4);
    memcpy(culled, v->culled, (size_t)v->n);
}

/* ---- coverage: the paper's sphere fill (paper/tex/voxelization.tex:24-27),
 * restated as a voxel-centre-in-ball test on the Q20 grid.  The code's own
 * fill loop is commented out (first_voxelize.glsl:54-58). ---------------- */
typedef struct { or_volume* v; } cov_ctx;

static void coverage_slice(void* p, long z) {
    or_volume* v = ((cov_ctx*)p)->v;
    int D = v->D;
    size_t base = (size_t)z * D * D;
    for (int b = 0; b < v->n; ++b) {
        if (v->culled[b]) continue;
        const int64_t* q = &v->q[3 * b];
        int xl, xh, yl, yh, zl, zh;
        board_axis_range(q[0], v->rq[b], D, &xl, &xh);
        board_axis_range(q[1], v->rq[b], D, &yl, &yh);
        board_axis_range(q[2], v->rq[b], D, &zl, &zh);
        if (z < zl || z > zh) continue;
        int64_t dz = (2 * (int64_t)z + 1) * HALF_Q20 - q[2];
        uint64_t dz2 = (uint64_t)(dz * dz);
        for (int y = yl; y <= yh; ++y) {
            int64_t dy = (2 * (int64_t)y + 1) * HALF_Q20 - q[1];
            uint64_t dyz = dz2 + (uint64_t)(dy * dy);
            for (int x = xl; x <= xh; ++x) {
                int64_t dx = (2 * (int64_t)x + 1) * HALF_Q20 - q[0];
                uint64_t d2 = dyz + (uint64_t)(dx * dx);
                if (d2 <= v->thr[b]) {
                    size_t i = base + (size_t)y * D + x;
                    v->count[i] += 1u;
                    v->dq[i] += v->dqb[b];
                }
            }
        }
    }
}

/* ---- sun-view nearest-surface map (first pass colour + depth) ---------- */
typedef struct { or_volume* v; f3* cv; } sun_ctx;

static void texel_range(const or_sun_frame* fr, float c, float r, int n, float lo_w,
                        int* a, int* b) {
    double span = (double)fr->hi - (double)fr->lo;
    double lo = ((double)c - (double)r - (double)fr->lo) / span * n - 0.5;
    double hi = ((double)c + (double)r - (double)fr->lo) / span * n - 0.5;
    (void)lo_w;
    long ia = (long)floor(lo) - 1, ib = (long)ceil(hi) + 1;
    if (ia < 0) ia = 0;
    if (ib > n - 1) ib = n - 1;
    *a = (int)ia;
    *b = (int)ib;
}

static void sunmap_row(void* p, long j) {
    sun_ctx* sc = (sun_ctx*)p;
    or_volume* v = sc->v;
    const or_sun_frame* fr = &v->frame;
    float yv = texel_y(fr, (int)j);
    uint64_t* row = v->keys + (size_t)j * fr->W;
    for (int b = 0; b < v->n; ++b) {
        f3 cv = sc->cv[b];
        float r = v->rad[b];
        int ja, jb;
        texel_range(fr, cv.y, r, fr->H, 0, &ja, &jb);
        if (j < ja || j > jb) continue;
        int ia, ib;
        texel_range(fr, cv.x, r, fr->W, 0, &ia, &ib);
        for (int i = ia; i <= ib; ++i) {
            float xv = texel_x(fr, i);
            float zs, depth;
            if (!sun_fragment(xv, yv, cv, r, fr->near_z, &zs, &depth)) continue;
            uint64_t key = ((uint64_t)f32_bits(depth) << 32) | (uint32_t)b;
            if (key < row[i]) row[i] = key;
        }
    }
}

/* World point of a sun-view texel's winning surface: eye + xv*s + yv*u + zs*(-f). */
static f3 sun_world(const or_sun_frame* fr, float xv, float yv, float zs) {
    float x = ((xv * fr->right[0] + yv * fr->up[0]) + zs * (-fr->fwd[0])) + fr->eye[0];
    float y = ((xv * fr->right[1] + yv * fr->up[1]) + zs * (-fr->fwd[1])) + fr->eye[1];
    float z = ((xv * fr->right[2] + yv * fr->up[2]) + zs * (-fr->fwd[2])) + fr->eye[2];
    return f3_make(x, y, z);
}

/* calculateVoxelIndex = ivec3(calculateVoxelLerp(p)) (second_voxelize.glsl:18-32):
 * truncation toward zero; stores outside [0,D) are dropped (imageStore). */
static int voxel_index(const or_volume* v, f3 p, int* ix, int* iy, int* iz) {
    float c[3] = {p.x, p.y, p.z};
    int o[3];
    float fd = (float)v->D;
    for (int a = 0; a < 3; ++a) {
        float t = (c[a] - v->wmin[a]) / v->range[a];
        float x = fd * t;
        if (!(x > -1.0f && x < fd)) return 0;
        o[a] = (int)x;
    }
    *ix = o[0]; *iy = o[1]; *iz = o[2];
    return 1;
}

/* second_voxelize.glsl:34-51 for one texel: 9 stores at p and at
 * p + stepSize*normalize(+-1,+-1,+-1).  The offset o = stepSize * 0.57735026
 * (float nearest 1/sqrt(3)), stepSize = min(voxelSize) (VoxelizeShader.cpp:128). */
static void highlight_texel(or_volume* v, f3 p, float o) {
    static const float sg[9][3] = {{0, 0, 0},  {1, 1, 1},  {1, 1, -1},  {1, -1, 1},  {1, -1, -1},
                                   {-1, 1, 1}, {-1, 1, -1}, {-1, -1, 1}, {-1, -1, -1}};
    for (int k = 0; k < 9; ++k) {
        f3 pk = p;
        if (k > 0) {
            pk.x = sg[k][0] > 0 ? p.x + o : p.x - o;
            pk.y = sg[k][1] > 0 ? p.y + o : p.y - o;
            pk.z = sg[k][2] > 0 ? p.z + o : p.z - o;
        }
        int ix, iy, iz;
        if (voxel_index(v, pk, &ix, &iy, &iz))
            v->mask[((size_t)iz * v->D + iy) * v->D + ix] = 1;
    }
}

/* Pass 2 alone over a given position map (W x H texels of xyzw, w > 0 =
 * written): the marks go to mask_out (D^3 bytes, cleared here); the volume's
 * own state is left unchanged. */
OR_API float or_highlight_offset(const or_volume* v);
OR_API void or_highlight_posmap(or_volume* v, const float* posmap, int W, int H,
                                uint8_t* mask_out) {
    uint8_t* keep = v->mask;
    memset(mask_out, 0, (size_t)v->D * v->D * v->D);
    v->mask = mask_out;
    float o = or_highlight_offset(v);
    for (size_t t = 0; t < (size_t)W * H; ++t) {
        const float* pm = posmap + t * 4;
        if (!(pm[3] > 0.0f)) continue;
        highlight_texel(v, f3_make(pm[0], pm[1], pm[2]), o);
    }
    v->mask = keep;
}

OR_API float or_highlight_offset(const or_volume* v) {
    float vs0 = v->range[0] / (float)v->D, vs1 = v->range[1] / (float)v->D,
          vs2 = v->range[2] / (float)v->D;
    float step = vs0 < vs1 ? vs0 : vs1;
    step = step < vs2 ? step : vs2;
    return step * 0.57735026f;
}

/* ---- mip pyramid: glGenerateMipmap (VoxelizeShader.cpp:105) as a 2x2x2 box
 * mean; child indices clamped to the level (only N=1 ever clamps). -------- */
typedef struct { or_volume* v; int l; } mip_ctx;

static void mip_slice(void* p, long z) {
    mip_ctx* mc = (mip_ctx*)p;
    or_volume* v = mc->v;
    int l = mc->l;
    int Nc = v->dims[l], Np = v->dims[l + 1];
    const real* src = v->rgba + v->offs[l] * 4;
    real* dst = v->rgba + v->offs[l + 1] * 4;
    for (int y = 0; y < Np; ++y)
        for (int x = 0; x < Np; ++x) {
            int cx[2] = {2 * x, 2 * x + 1}, cy[2] = {2 * y, 2 * y + 1},
                cz[2] = {2 * (int)z, 2 * (int)z + 1};
            for (int a = 0; a < 2; ++a) {
                if (cx[a] > Nc - 1) cx[a] = Nc - 1;
                if (cy[a] > Nc - 1) cy[a] = Nc - 1;
                if (cz[a] > Nc - 1) cz[a] = Nc - 1;
            }
            for (int ch = 0; ch < 4; ++ch) {
#define C(a, b, c) src[(((size_t)cz[c] * Nc + cy[b]) * Nc + cx[a]) * 4 + ch]
                real s = ((C(0, 0, 0) + C(1, 0, 0)) + (C(0, 1, 0) + C(1, 1, 0))) +
                         ((C(0, 0, 1) + C(1, 0, 1)) + (C(0, 1, 1) + C(1, 1, 1)));
#undef C
                dst[(((size_t)z * Np + y) * Np + x) * 4 + ch] = s * (real)0.125;
            }
        }
}

/* VoxelizeShader::voxelize (VoxelizeShader.cpp:18-31): clear, pass 1 (sun
 * map), pass 2 (highlights), coverage fill, level-0 assembly, mips.
 * Returns 0, or -1 when the sun direction is degenerate. */
OR_API int or_volume_voxelize(or_volume* v, const float dir[3], int W, int H, int nthreads) {
    if (or_sun_frame_make(v->pos, v->b0, v->b1, dir, W, H, &v->frame) != 0) return -1;
    int D = v->D;
    size_t n0 = (size_t)D * D * D;
    memset(v->count, 0, n0 * 4);
    memset(v->dq, 0, n0 * 4);
    memset(v->mask, 0, n0);
    if (v->mapW != W || v->mapH != H) {
        free(v->keys);
        free(v->posmap);
        v->keys = (uint64_t*)malloc((size_t)W * H * 8);
        v->posmap = (float*)malloc((size_t)W * H * 16);
        v->mapW = W;
        v->mapH = H;
    }
    memset(v->keys, 0xFF, (size_t)W * H * 8);
    memset(v->posmap, 0, (size_t)W * H * 16);
    /* pass 1: per texel nearest surface */
    f3* cv = (f3*)malloc(((size_t)v->n + 1) * sizeof(f3));
    for (int b = 0; b < v->n; ++b)
        cv[b] = sun_view_of(&v->frame, f3_make(v->cw[3 * b], v->cw[3 * b + 1], v->cw[3 * b + 2]));
    sun_ctx sc = {v, cv};
    or_parallel_for(H, nthreads, sunmap_row, &sc);
    /* pass 2: highlight stores (sequential: idempotent byte stores) */
    float o = or_highlight_offset(v);
    for (int j = 0; j < H; ++j) {
        float yv = texel_y(&v->frame, j);
        for (int i = 0; i < W; ++i) {
            uint64_t key = v->keys[(size_t)j * W + i];
            if (key == KEY_EMPTY) continue;
            int b = (int)(key & 0xFFFFFFFFu);
            float xv = texel_x(&v->frame, i);
            float zs, depth;
            sun_fragment(xv, yv, cv[b], v->rad[b], v->frame.near_z, &zs, &depth);
            f3 p = sun_world(&v->frame, xv, yv, zs);
            float* pm = v->posmap + ((size_t)j * W + i) * 4;
            pm[0] = p.x; pm[1] = p.y; pm[2] = p.z; pm[3] = 1.0f;
            highlight_texel(v, p, o);
        }
    }
    free(cv);
    /* coverage */
    cov_ctx cc = {v};
    or_parallel_for(D, nthreads, coverage_slice, &cc);
    /* level 0: R = density, G = light, B = count, A = occupancy */
    for (size_t i = 0; i < n0; ++i) {
        real* t = v->rgba + i * 4;
        t[0] = (real)v->dq[i] * (real)(1.0 / 65536.0);
        t[1] = v->mask[i] ? (real)1 : (real)0;
        t[2] = (real)v->count[i];
        t[3] = (v->count[i] > 0 || v->mask[i]) ? (real)1 : (real)0;
    }
    for (int l = 0; l + 1 < v->L; ++l) {
        mip_ctx mc = {v, l};
        or_parallel_for(v->dims[l + 1], nthreads, mip_slice, &mc);
    }
    return 0;
}

OR_API void or_volume_get_coverage(const or_volume* v, uint32_t* count, uint32_t* dq) {
    size_t n0 = (size_t)v->D * v->D * v->D;
    memcpy(count, v->count, n0 * 4);
    memcpy(dq, v->dq, n0 * 4);
}
OR_API void or_volume_get_mask(const or_volume* v, uint8_t* mask) {
    memcpy(mask, v->mask, (size_t)v->D * v->D * v->D);
}
OR_API void or_volume_get_sun_map(const or_volume* v, uint64_t* keys, float* pos) {
    memcpy(keys, v->keys, (size_t)v->mapW * v->mapH * 8);
    memcpy(pos, v->posmap, (size_t)v->mapW * v->mapH * 16);
}
OR_API void or_volume_get_frame(const or_volume* v, or_sun_frame* fr) { *fr = v->frame; }
/* Pyramid as doubles (total * 4). */
OR_API void or_volume_get_pyramid(const or_volume* v, double* out) {
    for (size_t i = 0; i < v->total * 4; ++i) out[i] = (double)v->rgba[i];
}
/* Replace the pyramid (total * 4 doubles), e.g. to evaluate the sampler or
 * the cone on a volume quantized like the product's BF16 storage. */
OR_API void or_volume_set_pyramid(or_volume* v, const double* in) {
    for (size_t i = 0; i < v->total * 4; ++i) v->rgba[i] = (real)in[i];
}

/* Recompute levels 1..L-1 from the current level 0 (for mip known-answer tests). */
OR_API void or_volume_rebuild_mips(or_volume* v, int nthreads) {
    for (int l = 0; l + 1 < v->L; ++l) {
        mip_ctx mc = {v, l};
        or_parallel_for(v->dims[l + 1], nthreads, mip_slice, &mc);
    }
}

/* ------------------------------------------------------------------ */
/* Sampler: textureLod with GL_LINEAR_MIPMAP_LINEAR (CloudVolume.cpp:19-23)   */
/* ------------------------------------------------------------------ */
#if defined(OR_REAL_IS_FLOAT)
#define RFLOOR floorf
#define RLOG2 log2f
#define REXP expf
#define RTAN tanf
#define RSQRT sqrtf
#else
#define RFLOOR floor
#define RLOG2 log2
#define REXP exp
#define RTAN tan
#define RSQRT sqrt
#endif

/* Trilinear at level l, voxel-space position v (level-0 voxel units).
 * Texel coords x = v * N_l / D - 0.5.  border = 1: taps outside the level read
 * 0 (the volume outside its box is empty); border = 0: CLAMP_TO_EDGE. */
static real sample_level(const or_volume* v, int l, const real p[3], int ch, int border) {
    int N = v->dims[l];
    real sc = (real)N / (real)v->D;
    int i0[3];
    real f[3];
    for (int a = 0; a < 3; ++a) {
        real x = p[a] * sc - (real)0.5;
        real fl = RFLOOR(x);
        f[a] = x - fl;
        i0[a] = (int)fl;
    }
    const real* base = v->rgba + v->offs[l] * 4;
    real c[2][2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                int ix = i0[0] + dx, iy = i0[1] + dy, iz = i0[2] + dz;
                real val;
                if (border) {
                    if (ix < 0 || iy < 0 || iz < 0 || ix >= N || iy >= N || iz >= N)
                        val = 0;
                    else
                        val = base[(((size_t)iz * N + iy) * N + ix) * 4 + ch];
                } else {
                    ix = ix < 0 ? 0 : (ix >= N ? N - 1 : ix);
                    iy = iy < 0 ? 0 : (iy >= N ? N - 1 : iy);
                    iz = iz < 0 ? 0 : (iz >= N ? N - 1 : iz);
                    val = base[(((size_t)iz * N + iy) * N + ix) * 4 + ch];
                }
                c[dz][dy][dx] = val;
            }
    real x00 = c[0][0][0] + f[0] * (c[0][0][1] - c[0][0][0]);
    real x10 = c[0][1][0] + f[0] * (c[0][1][1] - c[0][1][0]);
    real x01 = c[1][0][0] + f[0] * (c[1][0][1] - c[1][0][0]);
    real x11 = c[1][1][0] + f[0] * (c[1][1][1] - c[1][1][0]);
    real y0 = x00 + f[1] * (x10 - x00);
    real y1 = x01 + f[1] * (x11 - x01);
    return y0 + f[2] * (y1 - y0);
}

/* Quadrilinear: lod clamped to [0, L-1]; levels floor(lod) and floor(lod)+1
 * blended by the fractional part. */
static real sample_lod(const or_volume* v, const real p[3], real lod, int ch, int border) {
    real maxl = (real)(v->L - 1);
    if (!(lod > 0)) lod = 0;
    if (lod > maxl) lod = maxl;
    int l0 = (int)RFLOOR(lod);
    real fr = lod - (real)l0;
    real a = sample_level(v, l0, p, ch, border);
    if (fr > 0 && l0 + 1 < v->L) {
        real b = sample_level(v, l0 + 1, p, ch, border);
        return a + fr * (b - a);
    }
    return a;
}

OR_API double or_sample(const or_volume* v, const double p[3], double lod, int ch, int border) {
    real q[3] = {(real)p[0], (real)p[1], (real)p[2]};
    return (double)sample_lod(v, q, (real)lod, ch, border);
}

/* ------------------------------------------------------------------ */
/* Render parameters (mirror of the product's cg_render_params fields)  */
/* ------------------------------------------------------------------ */
typedef struct {
    int view_steps, sun_steps;
    float cone_half_angle, cone_initial_height, cone_min_radius, lod_offset, down_scaling;
    float density_scale, ambient;
    float sun_color[3];
    float transmittance_cutoff;
    int cone_mode;
    uint32_t noise_seed;
    int noise_octaves;
    float noise_frequency, noise_lacunarity, noise_gain;
    float noise_offset[3]; /* base-frequency lattice units (octaveOffsets) */
} or_params;

/* ---- sun cone -------------------------------------------------------
 * Mode 0 (transmittance): traceCone's schedule (conetrace_frag.glsl:64-79)
 * with the cone radius floored at cone_min_radius:
 *   h = h0; for i in 1..steps: r = max(h tan(a), rmin);
 *   lod = log2(max(1, 2r)) + lodOffset; R = density at v + h s;
 *   tau += R * r * voxel_world; h += r
 * (r and h in level-0 voxels).  Samples outside the box read 0; the loop stops
 * once a sample lies more than one coarsest texel outside (all further
 * samples are exactly 0).  Returns tau in world units.
 * Mode 1 (reference): the reference loop verbatim over the light channel
 * (the reference volume holds only second_voxelize's marks), clamp-to-edge,
 * coneAngle = 2*half-angle: sum += r_i * i / (steps * downScaling). */
static real sun_cone(const or_volume* v, const real p0[3], const real s[3], const or_params* P) {
    real h = (real)P->cone_initial_height;
    if (P->cone_mode == 1) {
        real tn = RTAN((real)(2.0f * P->cone_half_angle) / (real)2);
        real acc = 0;
        for (int i = 1; i <= P->sun_steps; ++i) {
            real rad = h * tn;
            real lod = RLOG2(rad * 2 > 1 ? rad * 2 : (real)1);
            real x[3] = {p0[0] + h * s[0], p0[1] + h * s[1], p0[2] + h * s[2]};
            real c = sample_lod(v, x, lod + (real)P->lod_offset, 1, 0);
            acc += c * (real)i / ((real)P->sun_steps * (real)P->down_scaling);
            h += rad;
        }
        return acc;
    }
    real tn = RTAN((real)P->cone_half_angle);
    real rmin = (real)P->cone_min_radius;
    real vw = (real)v->range[0] / (real)v->D;
    real E = (real)v->D / (real)v->dims[v->L - 1];
    real D = (real)v->D;
    real tau = 0, comp = 0; /* Neumaier */
    for (int i = 1; i <= P->sun_steps; ++i) {
        real rad = h * tn;
        if (rad < rmin) rad = rmin;
        real lod = RLOG2(rad * 2 > 1 ? rad * 2 : (real)1) + (real)P->lod_offset;
        real x[3] = {p0[0] + h * s[0], p0[1] + h * s[1], p0[2] + h * s[2]};
        if (x[0] < -E || x[1] < -E || x[2] < -E || x[0] > D + E || x[1] > D + E || x[2] > D + E)
            break;
        real R = sample_lod(v, x, lod, 0, 1);
        real term = R * rad * vw;
        real t = tau + term;
        if ((tau >= 0 ? tau : -tau) >= (term >= 0 ? term : -term))
            comp += (tau - t) + term;
        else
            comp += (term - t) + tau;
        tau = t;
        h += rad;
    }
    return tau + comp;
}

OR_API double or_trace_cone(const or_volume* v, const double p[3], const double dir[3],
                            const or_params* P) {
    real q[3] = {(real)p[0], (real)p[1], (real)p[2]};
    /* direction = normalize(direction) (conetrace_frag.glsl:65) */
    double n = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    real s[3] = {(real)(dir[0] / n), (real)(dir[1] / n), (real)(dir[2] / n)};
    return (double)sun_cone(v, q, s, P);
}

/* ------------------------------------------------------------------ */
/* Hash value-noise fBm (replaces the noise texture, ConeTraceShader.cpp:127-159;
 * fBm structure of noise3D, conetrace_frag.glsl:103-120).                     */
/* ------------------------------------------------------------------ */
/* PCG3D (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020). */
OR_API void or_pcg3d(uint32_t v[3]) {
    v[0] = v[0] * 1664525u + 1013904223u;
    v[1] = v[1] * 1664525u + 1013904223u;
    v[2] = v[2] * 1664525u + 1013904223u;
    v[0] += v[1] * v[2];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
    v[0] ^= v[0] >> 16;
    v[1] ^= v[1] >> 16;
    v[2] ^= v[2] >> 16;
    v[0] += v[1] * v[2];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
}

/* Lattice value in [0,1): 24 high bits of pcg3d(x + k, y + (k ^ c1), z + (k ^ c2)).x
 * with the octave key k = seed * 0x9E3779B9 + octave * 0x85EBCA6B + 1. */
OR_API double or_lattice(int ix, int iy, int iz, uint32_t seed, int octave) {
    uint32_t k = seed * 0x9E3779B9u + (uint32_t)octave * 0x85EBCA6Bu + 1u;
    uint32_t h[3] = {(uint32_t)ix + k, (uint32_t)iy + (k ^ 0x68E31DA4u),
                     (uint32_t)iz + (k ^ 0xB5297A4Du)};
    or_pcg3d(h);
    return (double)(h[0] >> 8) * (1.0 / 16777216.0);
}

static real lattice_r(int ix, int iy, int iz, uint32_t seed, int octave) {
    uint32_t k = seed * 0x9E3779B9u + (uint32_t)octave * 0x85EBCA6Bu + 1u;
    uint32_t h[3] = {(uint32_t)ix + k, (uint32_t)iy + (k ^ 0x68E31DA4u),
                     (uint32_t)iz + (k ^ 0xB5297A4Du)};
    or_pcg3d(h);
    return (real)(h[0] >> 8) * (real)(1.0 / 16777216.0);
}

/* Value noise: trilinear over the lattice with smoothstep weights w = f^2 (3-2f). */
static real value_noise(const real x[3], uint32_t seed, int octave) {
    int i[3];
    real w[3];
    for (int a = 0; a < 3; ++a) {
        real fl = RFLOOR(x[a]);
        real f = x[a] - fl;
        i[a] = (int)fl;
        w[a] = f * f * ((real)3 - (real)2 * f);
    }
    real c[2][2][2];
    for (int dz = 0; dz < 2; ++dz)
        for (int dy = 0; dy < 2; ++dy)
            for (int dx = 0; dx < 2; ++dx)
                c[dz][dy][dx] = lattice_r(i[0] + dx, i[1] + dy, i[2] + dz, seed, octave);
    real x00 = c[0][0][0] + w[0] * (c[0][0][1] - c[0][0][0]);
    real x10 = c[0][1][0] + w[0] * (c[0][1][1] - c[0][1][0]);
    real x01 = c[1][0][0] + w[0] * (c[1][0][1] - c[1][0][0]);
    real x11 = c[1][1][0] + w[0] * (c[1][1][1] - c[1][1][0]);
    real y0 = x00 + w[1] * (x10 - x00);
    real y1 = x01 + w[1] * (x11 - x01);
    return y0 + w[2] * (y1 - y0);
}

/* fBm = sum_k gain^k noise_k((p * freq + offset) * lac^k) / sum_k gain^k; 1 when
 * octaves = 0.  The offset is the reference's per-octave octaveOffsets = windVel *
 * runTime (ConeTraceShader.cpp:55-61), added to the base-frequency noise
 * coordinate before the octave's frequency step (conetrace_frag.glsl:110); it is
 * applied here as the world shift offset / freq. */
static real fbm(const real p[3], const or_params* P) {
    if (P->noise_octaves <= 0) return (real)1;
    real amp = 1, norm = 0, sum = 0, f = (real)P->noise_frequency;
    real q[3];
    for (int a = 0; a < 3; ++a)
        q[a] = p[a] + (real)((double)P->noise_offset[a] / (double)P->noise_frequency);
    for (int k = 0; k < P->noise_octaves; ++k) {
        real x[3] = {q[0] * f, q[1] * f, q[2] * f};
        sum += amp * value_noise(x, P->noise_seed, k);
        norm += amp;
        amp *= (real)P->noise_gain;
        f *= (real)P->noise_lacunarity;
    }
    return sum / norm;
}

OR_API double or_fbm(const double p[3], const or_params* P) {
    real q[3] = {(real)p[0], (real)p[1], (real)p[2]};
    return (double)fbm(q, P);
}

/* ------------------------------------------------------------------ */
/* View march (build-defined; replaces the per-billboard fragment shading of
 * conetrace_frag.glsl:122-201 and the back-to-front blend, main.cpp:94-95).   */
/* ------------------------------------------------------------------ */
typedef struct {
    double eye[3], target[3], up[3];
    double fov_y_degrees;
    int width, height;
} or_camera;

typedef struct {
    const or_volume* v;
    const or_camera* cam;
    const or_params* P;
    real f[3], s[3], u[3];
    real tanh, aspect;
    real sun[3];
    int x0, y0, w, h;
    double* out;
    int64_t* stats; /* per row: [view samples, sun cones] */
} render_ctx;

static void normalize_r(real v[3]) {
    real n = RSQRT(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] /= n; v[1] /= n; v[2] /= n;
}

static void render_pixel(const render_ctx* rc, int px, int py, double* o, int64_t* st) {
    const or_volume* v = rc->v;
    const or_params* P = rc->P;
    const or_camera* cam = rc->cam;
    real ndx = ((real)2 * ((real)px + (real)0.5) / (real)cam->width - (real)1) * rc->tanh * rc->aspect;
    real ndy = ((real)1 - (real)2 * ((real)py + (real)0.5) / (real)cam->height) * rc->tanh;
    real d[3];
    for (int a = 0; a < 3; ++a) d[a] = rc->f[a] + ndx * rc->s[a] + ndy * rc->u[a];
    normalize_r(d);
    real e[3] = {(real)cam->eye[0], (real)cam->eye[1], (real)cam->eye[2]};
    /* slab test against the world box */
    real tmin = -1e30, tmax = 1e30;
    for (int a = 0; a < 3; ++a) {
        real lo = (real)v->wmin[a], hi = (real)v->wmax[a];
        if (d[a] == 0) {
            if (e[a] < lo || e[a] > hi) { tmin = 1; tmax = 0; }
            continue;
        }
        real inv = (real)1 / d[a];
        real t0 = (lo - e[a]) * inv, t1 = (hi - e[a]) * inv;
        if (t0 > t1) { real tt = t0; t0 = t1; t1 = tt; }
        if (t0 > tmin) tmin = t0;
        if (t1 < tmax) tmax = t1;
    }
    real tin = tmin > 0 ? tmin : 0;
    real tout = tmax;
    o[0] = o[1] = o[2] = o[3] = 0;
    if (!(tout > tin)) return;
    int Nv = P->view_steps;
    real dt = (tout - tin) / (real)Nv;
    real Dr = (real)v->D;
    real vox = Dr / (real)v->range[0]; /* voxels per world unit */
    real pixk = rc->tanh / (real)cam->height * vox;
    real sigma = (real)P->density_scale;
    real amb = (real)P->ambient;
    real T = 1, C = 0, Cc = 0;
    for (int k = 0; k < Nv; ++k) {
        real t = tin + ((real)k + (real)0.5) * dt;
        real p[3] = {e[0] + t * d[0], e[1] + t * d[1], e[2] + t * d[2]};
        real vp[3];
        for (int a = 0; a < 3; ++a) vp[a] = (p[a] - (real)v->wmin[a]) / (real)v->range[a] * Dr;
        real rp = t * pixk;
        real lod = RLOG2(rp * 2 > 1 ? rp * 2 : (real)1);
        real R = sample_lod(v, vp, lod, 0, 1);
        st[0]++;
        if (!(R > 0)) continue;
        real rho = R * fbm(p, P);
        if (!(rho > 0)) continue;
        real alpha = (real)1 - REXP(-sigma * rho * dt);
        real G = sample_lod(v, vp, lod, 1, 1);
        real tau = sun_cone(v, vp, rc->sun, P);
        st[1]++;
        real Ts = REXP(-sigma * tau);
        real L = Ts * (amb + ((real)1 - amb) * G);
        real term = T * alpha * L;
        real tt = C + term;
        if ((C >= 0 ? C : -C) >= (term >= 0 ? term : -term))
            Cc += (C - tt) + term;
        else
            Cc += (term - tt) + C;
        C = tt;
        T *= (real)1 - alpha;
        if (T < (real)P->transmittance_cutoff) break;
    }
    C += Cc;
    o[0] = (double)(C * (real)P->sun_color[0]);
    o[1] = (double)(C * (real)P->sun_color[1]);
    o[2] = (double)(C * (real)P->sun_color[2]);
    o[3] = (double)((real)1 - T);
}

static void render_row(void* p, long r) {
    render_ctx* rc = (render_ctx*)p;
    int py = rc->y0 + (int)r;
    int64_t* st = rc->stats ? rc->stats + 2 * r : NULL;
    int64_t dummy[2];
    if (!st) st = dummy;
    st[0] = st[1] = 0;
    for (int i = 0; i < rc->w; ++i) {
        double* o = rc->out + ((size_t)r * rc->w + i) * 4;
        render_pixel(rc, rc->x0 + i, py, o, st);
    }
}

static void camera_basis(const or_camera* cam, real f[3], real s[3], real u[3]) {
    for (int a = 0; a < 3; ++a) f[a] = (real)(cam->target[a] - cam->eye[a]);
    normalize_r(f);
    real up[3] = {(real)cam->up[0], (real)cam->up[1], (real)cam->up[2]};
    s[0] = f[1] * up[2] - up[1] * f[2];
    s[1] = f[2] * up[0] - up[2] * f[0];
    s[2] = f[0] * up[1] - up[0] * f[1];
    normalize_r(s);
    u[0] = s[1] * f[2] - f[1] * s[2];
    u[1] = s[2] * f[0] - f[2] * s[0];
    u[2] = s[0] * f[1] - f[0] * s[1];
}

/* Render the rectangle [x0, x0+w) x [y0, y0+h) of the camera's image into out
 * (w*h*4 doubles).  stats (h*2, may be NULL) receives per-row counts of view
 * samples and sun cones.  Returns 0. */
OR_API int or_render(const or_volume* v, const or_camera* cam, const or_params* P,
                     const float sun_dir[3], int x0, int y0, int w, int h, double* out,
                     int64_t* stats, int nthreads) {
    render_ctx rc;
    rc.v = v;
    rc.cam = cam;
    rc.P = P;
    camera_basis(cam, rc.f, rc.s, rc.u);
    rc.tanh = RTAN((real)(cam->fov_y_degrees * 3.14159265358979323846 / 180.0) / (real)2);
    rc.aspect = (real)cam->width / (real)cam->height;
    real sd[3] = {(real)sun_dir[0], (real)sun_dir[1], (real)sun_dir[2]};
    normalize_r(sd);
    rc.sun[0] = sd[0]; rc.sun[1] = sd[1]; rc.sun[2] = sd[2];
    rc.x0 = x0; rc.y0 = y0; rc.w = w; rc.h = h;
    rc.out = out;
    rc.stats = stats;
    or_parallel_for(h, nthreads, render_row, &rc);
    return 0;
}

OR_API int or_real_bytes(void) { return (int)sizeof(real); }

/* ------------------------------------------------------------------ */
/* Compat render: the reference's own image formation, one camera-facing   */
/* billboard per board shaded by conetrace_frag.glsl:122-201 and blended    */
/* back to front (ConeTraceShader::coneTrace, ConeTraceShader.cpp:15-82;     */
/* sortBoards, CloudVolume.cpp:65-82; blend state main.cpp:94-95), restated  */
/* per pixel:                                                               */
/*  - quad: c + r (x s + y u), x, y in [-1, 1] (billboard_vert_instanced.glsl */
/*    with Library::createQuad), camera-facing, so every pixel's fragment is  */
/*    the plane point e + z d (z = (c - e).f, d the pixel ray with d.f = 1);  */
/*    the quad is drawn only when near < z < 2500 (Camera.cpp:59);           */
/*  - fragment: the shader's noise march and traceCone, with lightPos far     */
/*    along the sun direction (dir = sun) and the noise map supplied as a    */
/*    decoded 32^3 RGBA table (REPEAT, LINEAR; octave k adds the scalar      */
/*    octaveOffsets[k], k < 3, else 0 -- the shader indexes a vec3);         */
/*  - blend: source clamped to [0, 1] (fixed-point target), then            */
/*    C = a src + (1 - a) C for RGB and A = a a + (1 - a) A over the clear    */
/*    colour, boards in descending (distance to the eye, index) order.       */
/* ------------------------------------------------------------------ */
typedef struct {
    int show_quad, do_noise, do_cone_trace;
    float step_size, noise_opacity;
    int num_octaves;
    float freq_step, pers_step, adjust_size;
    int min_noise_steps, max_noise_steps;
    float min_noise_color, noise_color_scale;
    float octave_offsets[3];
    uint32_t noise_seed;
    int vct_steps;
    float vct_cone_angle, vct_cone_initial_height, vct_lod_offset, vct_down_scaling;
    float clear_color[4];
    float near_plane;
    float transmittance_cutoff;
} or_compat_params;

#define CN 32 /* noise map edge (ConeTraceShader.cpp:12, initNoiseMap(32)) */

static uint64_t splitmix_next(uint64_t* st) {
    uint64_t z = (*st += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Largest c >= 0 with c^2 * S <= 16384 * g^2 (= floor(128 |g| / sqrt(S))). */
static int snorm_component(int g, int64_t S) {
    if (S == 0) return 0;
    int64_t G2 = (int64_t)16384 * g * g;
    int c = (int)floor(sqrt((double)G2 / (double)S));
    while (c > 0 && (int64_t)c * c * S > G2) --c;
    while ((int64_t)(c + 1) * (c + 1) * S <= G2) ++c;
    if (c > 127) c = 127;
    return g < 0 ? -c : c;
}

/* The 32^3 noise map of initNoiseMap (ConeTraceShader.cpp:127-159) from a
 * seeded stream: alpha a = uniform integer in [-128, 127]; RGB = the unit
 * "gradient" with the reference's operator precedence,
 * g_x = d(x+1) - d(x-1) / 0.5 with d = a / 128 (neighbours wrap), i.e. the
 * integer G = a(x+1) - 2 a(x-1), stored as trunc(128 n) with n = G / |G|
 * (0 where G = 0, at most 127 in magnitude), evaluated exactly; decoded as
 * GL_RGBA8_SNORM: max(c / 127, -1).  out: 32^3 x 4 floats, x fastest. */
OR_API void or_compat_noise_map(uint32_t seed, float* out) {
    static int8_t a[CN * CN * CN];
    uint64_t st = (uint64_t)seed * 0x2545F4914F6CDD1DULL + 0x632BE59BD9B4E019ULL;
    for (int i = 0; i < CN * CN * CN; ++i) a[i] = (int8_t)((int)(splitmix_next(&st) >> 56) - 128);
#define WRAP(i) (((i) % CN + CN) % CN)
#define AT(x, y, z) a[WRAP(x) + WRAP(y) * CN + WRAP(z) * CN * CN]
    for (int z = 0; z < CN; ++z)
        for (int y = 0; y < CN; ++y)
            for (int x = 0; x < CN; ++x) {
                int g[3] = {AT(x + 1, y, z) - 2 * AT(x - 1, y, z),
                            AT(x, y + 1, z) - 2 * AT(x, y - 1, z),
                            AT(x, y, z + 1) - 2 * AT(x, y, z - 1)};
                int64_t S = (int64_t)g[0] * g[0] + (int64_t)g[1] * g[1] + (int64_t)g[2] * g[2];
                float* o = out + 4 * (size_t)(x + y * CN + z * CN * CN);
                for (int k = 0; k < 3; ++k) o[k] = (float)snorm_component(g[k], S) / 127.0f;
                float av = (float)AT(x, y, z) / 127.0f;
                o[3] = av < -1.0f ? -1.0f : av;
            }
#undef AT
#undef WRAP
}

/* texture(noiseMap, q): LINEAR with REPEAT at normalised coordinates. */
static void noise_tap(const float* tab, const real q[3], real out[4]) {
    int i0[3], i1[3];
    real f[3];
    for (int a = 0; a < 3; ++a) {
        real x = q[a] * (real)CN - (real)0.5;
        real fl = RFLOOR(x);
        f[a] = x - fl;
        long long ii = (long long)fl;
        int m = (int)(((ii % CN) + CN) % CN);
        i0[a] = m;
        i1[a] = (m + 1) % CN;
    }
    for (int ch = 0; ch < 4; ++ch) {
        real c[2][2][2];
        for (int dz = 0; dz < 2; ++dz)
            for (int dy = 0; dy < 2; ++dy)
                for (int dx = 0; dx < 2; ++dx) {
                    int x = dx ? i1[0] : i0[0], y = dy ? i1[1] : i0[1], z = dz ? i1[2] : i0[2];
                    c[dz][dy][dx] = (real)tab[4 * (size_t)(x + y * CN + z * CN * CN) + ch];
                }
        real x00 = c[0][0][0] + f[0] * (c[0][0][1] - c[0][0][0]);
        real x10 = c[0][1][0] + f[0] * (c[0][1][1] - c[0][1][0]);
        real x01 = c[1][0][0] + f[0] * (c[1][0][1] - c[1][0][0]);
        real x11 = c[1][1][0] + f[0] * (c[1][1][1] - c[1][1][0]);
        real y0 = x00 + f[1] * (x10 - x00);
        real y1 = x01 + f[1] * (x11 - x01);
        out[ch] = y0 + f[2] * (y1 - y0);
    }
}

typedef struct {
    const or_volume* v;
    const or_camera* cam;
    const or_compat_params* P;
    const float* noise;
    real f[3], s[3], u[3], e[3];
    real tanh, aspect, sun[3];
    const int* order; /* boards back to front */
    int n_order;
    const real* cw; /* per board: centre xyz, radius, z */
    int W, H;
    double* out;
} compat_ctx;

static real dot3(const real a[3], const real b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static real sat(real x) { return x < 0 ? 0 : (x > 1 ? 1 : x); }

/* traceCone (conetrace_frag.glsl:64-79) from level-0 voxel position vp along
 * the unit direction dir, over the light channel with CLAMP_TO_EDGE. */
static real compat_trace_cone(const compat_ctx* cc, const real vp[3]) {
    const or_compat_params* P = cc->P;
    real h = (real)P->vct_cone_initial_height, acc = 0;
    real th = RTAN((real)P->vct_cone_angle / (real)2);
    for (int i = 1; i <= P->vct_steps; ++i) {
        real cr = h * th;
        real lod = RLOG2(2 * cr > 1 ? 2 * cr : (real)1);
        real q[3] = {vp[0] + h * cc->sun[0], vp[1] + h * cc->sun[1], vp[2] + h * cc->sun[2]};
        real smp = sample_lod(cc->v, q, lod + (real)P->vct_lod_offset, 1, 0);
        acc += smp * (real)i / ((real)P->vct_steps * (real)P->vct_down_scaling);
        h += cr;
    }
    return acc;
}

/* The fragment shader at plane point fp (quad texture coordinate ft) of the
 * board with centre c and radius r; returns 0 when it discards. */
static int compat_fragment(const compat_ctx* cc, const real fp[3], const real ft[2],
                           const real c[3], real r, real o[4]) {
    const or_compat_params* P = cc->P;
    real dc[3] = {fp[0] - c[0], fp[1] - c[1], fp[2] - c[2]};
    if (P->show_quad) {
        real sc = RSQRT(dot3(dc, dc)) / r;
        real t = 1 - sc * sc;
        sc = RSQRT(t > 0 ? t : (real)0);
        o[0] = o[1] = o[2] = o[3] = sc;
        if (ft[0] < (real)0.01f || ft[1] < (real)0.01f || ft[0] > (real)0.99f || ft[1] > (real)0.99f)
            o[0] = o[1] = o[2] = o[3] = 1;
        return 1;
    }
    const real back[3] = {-cc->f[0], -cc->f[1], -cc->f[2]};
    if (P->do_noise) {
        real A = dot3(back, back), B = 2 * dot3(dc, back), C = dot3(dc, dc) - r * r;
        real disc = B * B - 4 * A * C;
        if (disc < (real)0.01f) return 0;
        real sq = RSQRT(disc);
        real tn = (-B - sq) / (2 * A), tf = (-B + sq) / (2 * A);
        real wn[3], wf[3], ut[3], ct[3], dl[3];
        real k = (real)1 / (real)P->adjust_size;
        for (int a = 0; a < 3; ++a) {
            wn[a] = fp[a] + back[a] * tn;
            wf[a] = fp[a] + back[a] * tf;
            ut[a] = (wn[a] - c[a]) / r;
            ct[a] = wn[a] * k;
        }
        real len2 = 0;
        for (int a = 0; a < 3; ++a) {
            real dd = wf[a] * k - ct[a];
            len2 += dd * dd;
        }
        real is = RSQRT(len2) / (real)P->step_size;
        real span = (real)(P->max_noise_steps - P->min_noise_steps);
        is = (is < span ? is : span) + (real)P->min_noise_steps;
        for (int a = 0; a < 3; ++a) dl[a] = (wf[a] * k - ct[a]) / (is - 1);
        real oa = (real)P->noise_opacity / (is - 1), la = (real)1 / (is - 1);
        real ro = 0, rl = 0;
        for (int i = 0; (real)i < is; ++i) {
            real nv[4] = {0, 0, 0, 0}, fr = 1, pe = 1;
            for (int oc = 0; oc < P->num_octaves; ++oc) {
                real off = oc < 3 ? (real)P->octave_offsets[oc] : 0;
                real q[3] = {(ct[0] + off) * fr, (ct[1] + off) * fr, (ct[2] + off) * fr};
                real tv[4];
                noise_tap(cc->noise, q, tv);
                for (int ch = 0; ch < 4; ++ch) nv[ch] += pe * tv[ch];
                fr *= (real)P->freq_step;
                pe *= (real)P->pers_step;
            }
            nv[3] = nv[3] < 0 ? -nv[3] : nv[3];
            real un = RSQRT(dot3(ut, ut));
            for (int a = 0; a < 3; ++a) nv[a] += ut[a] / un;
            ro += nv[3] * (1 - dot3(ut, ut));
            rl += sat(nv[1] * (real)0.5 + (real)0.5);
            for (int a = 0; a < 3; ++a) {
                ct[a] += dl[a];
                ut[a] += dl[a];
            }
        }
        real col = (real)P->min_noise_color + (real)P->noise_color_scale * rl * la;
        real tx = ft[0] - (real)0.5, ty = ft[1] - (real)0.5;
        real alpha = 1 - RSQRT(tx * tx + ty * ty) * 2;
        ro = sat(ro * oa);
        o[0] = o[1] = o[2] = col;
        o[3] = ro * alpha;
    }
    if (P->do_cone_trace) {
        real sc = RSQRT(dot3(dc, dc)) / r;
        real t = 1 - sc * sc;
        sc = RSQRT(t > 0 ? t : (real)0);
        if (sc < (real)0.01f) return 0;
        const or_volume* v = cc->v;
        real vp[3];
        for (int a = 0; a < 3; ++a) {
            real pos = fp[a] + back[a] * r * sc;
            vp[a] = (real)v->D * ((pos - (real)v->wmin[a]) / (real)v->range[a]);
        }
        real ind = compat_trace_cone(cc, vp);
        if (P->do_noise) {
            o[0] *= ind;
            o[1] *= ind;
            o[2] *= ind;
        } else {
            o[0] = o[1] = o[2] = o[3] = ind;
        }
    }
    return 1;
}

static void compat_row(void* p, long row) {
    const compat_ctx* cc = (const compat_ctx*)p;
    const or_compat_params* P = cc->P;
    for (int px = 0; px < cc->W; ++px) {
        real ndx = ((real)2 * ((real)px + (real)0.5) / (real)cc->W - (real)1) * cc->tanh * cc->aspect;
        real ndy = ((real)1 - (real)2 * ((real)row + (real)0.5) / (real)cc->H) * cc->tanh;
        real d[3];
        for (int a = 0; a < 3; ++a) d[a] = cc->f[a] + ndx * cc->s[a] + ndy * cc->u[a];
        real C[4] = {(real)P->clear_color[0], (real)P->clear_color[1], (real)P->clear_color[2],
                     (real)P->clear_color[3]};
        if (P->show_quad || P->do_noise || P->do_cone_trace)
            for (int k = 0; k < cc->n_order; ++k) {
                const real* b = cc->cw + 5 * cc->order[k];
                real z = b[4], r = b[3];
                real fp[3], dc[3];
                for (int a = 0; a < 3; ++a) {
                    fp[a] = cc->e[a] + z * d[a];
                    dc[a] = fp[a] - b[a];
                }
                real x = dot3(dc, cc->s) / r, y = dot3(dc, cc->u) / r;
                if (!(x >= -1 && x <= 1 && y >= -1 && y <= 1)) continue;
                real ft[2] = {(x + 1) / 2, (y + 1) / 2};
                real o[4];
                if (!compat_fragment(cc, fp, ft, b, r, o)) continue;
                for (int ch = 0; ch < 4; ++ch) o[ch] = sat(o[ch]);
                real al = o[3];
                for (int ch = 0; ch < 3; ++ch) C[ch] = al * o[ch] + (1 - al) * C[ch];
                C[3] = al * al + (1 - al) * C[3];
            }
        double* out = cc->out + ((size_t)row * cc->W + px) * 4;
        for (int ch = 0; ch < 4; ++ch) out[ch] = (double)C[ch];
    }
}

static const real* g_sort_keys;
static int compat_cmp(const void* a, const void* b) {
    int i = *(const int*)a, j = *(const int*)b;
    real di = g_sort_keys[i], dj = g_sort_keys[j];
    if (di != dj) return di > dj ? -1 : 1; /* farthest first */
    return i > j ? -1 : (i < j ? 1 : 0);
}

/* The compat image of the volume's boards (world centres and radii as
 * uploaded) seen by cam, sun direction sun_dir (light channel of the
 * pyramid for the cone), noise map tab (or_compat_noise_map).  out: W*H*4
 * doubles, row 0 = top. */
OR_API int or_compat_render(const or_volume* v, const or_camera* cam, const or_compat_params* P,
                            const float sun_dir[3], const float* tab, double* out, int nthreads) {
    compat_ctx cc;
    memset(&cc, 0, sizeof(cc));
    cc.v = v;
    cc.cam = cam;
    cc.P = P;
    cc.noise = tab;
    camera_basis(cam, cc.f, cc.s, cc.u);
    for (int a = 0; a < 3; ++a) cc.e[a] = (real)cam->eye[a];
    cc.tanh = RTAN((real)(cam->fov_y_degrees * 3.14159265358979323846 / 180.0) / (real)2);
    cc.aspect = (real)cam->width / (real)cam->height;
    real sd[3] = {(real)sun_dir[0], (real)sun_dir[1], (real)sun_dir[2]};
    normalize_r(sd);
    for (int a = 0; a < 3; ++a) cc.sun[a] = sd[a];
    cc.W = cam->width;
    cc.H = cam->height;
    cc.out = out;
    int n = v->n;
    real* cw = (real*)malloc((size_t)(n > 0 ? n : 1) * 5 * sizeof(real));
    real* key = (real*)malloc((size_t)(n > 0 ? n : 1) * sizeof(real));
    int* order = (int*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    int m = 0;
    for (int b = 0; b < n; ++b) {
        real c[3] = {(real)v->cw[3 * b], (real)v->cw[3 * b + 1], (real)v->cw[3 * b + 2]};
        real dc[3] = {c[0] - cc.e[0], c[1] - cc.e[1], c[2] - cc.e[2]};
        real z = dot3(dc, cc.f);
        for (int a = 0; a < 3; ++a) cw[5 * b + a] = c[a];
        cw[5 * b + 3] = (real)v->rad[b];
        cw[5 * b + 4] = z;
        key[b] = RSQRT(dot3(dc, dc));
        if (z > (real)P->near_plane && z < (real)2500 && v->rad[b] > 0) order[m++] = b;
    }
    g_sort_keys = key;
    qsort(order, (size_t)m, sizeof(int), compat_cmp);
    cc.order = order;
    cc.n_order = m;
    cc.cw = cw;
    or_parallel_for(cc.H, nthreads, compat_row, &cc);
    free(cw);
    free(key);
    free(order);
    return 0;
}

/* ------------------------------------------------------------------ */
/* MLP sun-transmittance surrogate in FP64 (build-defined; the reference    */
/* has no learned part).  Parameter layout: W1[64][16] b1[64] W2[64][64]    */
/* b2[64] W3[64][64] b3[64] W4[1][64] b4[1] (9473 values, W as [out][in]).   */
/* ------------------------------------------------------------------ */
#define M_W1 0
#define M_B1 1024
#define M_W2 1088
#define M_B2 5184
#define M_W3 5248
#define M_B3 9344
#define M_W4 9408
#define M_B4 9472
#define M_NPARAM 9473

/* f[3i+k] = level (lb+i) trilinear density (border 0) at
 * p + (h0 + (k + 0.5) * 2^(lb+i)) * s; f[12..14] = p / D; f[15] = s.y. */
OR_API void or_mlp_features(const or_volume* v, const double p[3], const double s[3], int lb,
                            double h0, double out[16]) {
    for (int i = 0; i < 4; ++i) {
        int lv = lb + i;
        int l = lv < 0 ? 0 : (lv > v->L - 1 ? v->L - 1 : lv);
        double span = (double)(1 << lv);
        for (int k = 0; k < 3; ++k) {
            double d = h0 + ((double)k + 0.5) * span;
            real q[3] = {(real)(p[0] + d * s[0]), (real)(p[1] + d * s[1]), (real)(p[2] + d * s[2])};
            out[3 * i + k] = (double)sample_level(v, l, q, 0, 1);
        }
    }
    for (int a = 0; a < 3; ++a) out[12 + a] = p[a] / (double)v->D;
    out[15] = s[1];
}

static double silu_d(double z) { return z / (1.0 + exp(-z)); }
static double silu_grad_d(double z) {
    double s = 1.0 / (1.0 + exp(-z));
    return s * (1.0 + z * (1.0 - s));
}

static void mlp_layer(const double* W, const double* b, const double* x, int nin, double* z) {
    for (int o = 0; o < 64; ++o) {
        double acc = b[o];
        for (int i = 0; i < nin; ++i) acc += W[o * nin + i] * x[i];
        z[o] = acc;
    }
}

/* Hidden layer l (0-based) of the parameter vector: weights, bias, fan-in. */
static const double* mlp_w(const double* P, int l) { return P + (l == 0 ? M_W1 : (l == 1 ? M_W2 : M_W3)); }
static const double* mlp_b(const double* P, int l) { return P + (l == 0 ? M_B1 : (l == 1 ? M_B2 : M_B3)); }
static int mlp_nin(int l) { return l == 0 ? 16 : 64; }
static int mlp_woff(int l) { return l == 0 ? M_W1 : (l == 1 ? M_W2 : M_W3); }
static int mlp_boff(int l) { return l == 0 ? M_B1 : (l == 1 ? M_B2 : M_B3); }

/* Normalised output y of one row of raw features f through `layers` (1..3)
 * hidden layers; the output layer (W4, b4) reads the last one. */
OR_API double or_mlp_forward(const double* P, const double* mu, const double* sd,
                             const double f[16], int layers) {
    double a[64], z[64];
    for (int j = 0; j < 16; ++j) a[j] = (f[j] - mu[j]) / sd[j];
    for (int l = 0; l < layers; ++l) {
        mlp_layer(mlp_w(P, l), mlp_b(P, l), a, mlp_nin(l), z);
        for (int o = 0; o < 64; ++o) a[o] = silu_d(z[o]);
    }
    double y = P[M_B4];
    for (int i = 0; i < 64; ++i) y += P[M_W4 + i] * a[i];
    return y;
}

/* Mean over n rows of (exp(-sigma*scale*softplus(y)) - exp(-sigma*tau))^2 and
 * its gradient with respect to the 9473 parameters (grad, zeroed here; the
 * blocks of unused hidden layers stay 0) for a network of `layers` (1..3)
 * hidden layers.  The predicted optical depth is scale * softplus(y). */
OR_API double or_mlp_loss_grad(const double* P, const double* mu, const double* sd,
                               double tau_scale, double sigma, const double* feats,
                               const double* tau, int n, double* grad, int layers) {
    for (int i = 0; i < M_NPARAM; ++i) grad[i] = 0.0;
    double loss = 0.0;
    for (int r = 0; r < n; ++r) {
        /* h[0] = x (16 wide), h[l+1] = silu(z[l]) */
        double h[4][64], z[3][64];
        for (int j = 0; j < 16; ++j) h[0][j] = (feats[r * 16 + j] - mu[j]) / sd[j];
        for (int l = 0; l < layers; ++l) {
            mlp_layer(mlp_w(P, l), mlp_b(P, l), h[l], mlp_nin(l), z[l]);
            for (int o = 0; o < 64; ++o) h[l + 1][o] = silu_d(z[l][o]);
        }
        const double* hl = h[layers];
        double y = P[M_B4];
        for (int i = 0; i < 64; ++i) y += P[M_W4 + i] * hl[i];
        double k = sigma * tau_scale;
        double sp = (y > 0 ? y : 0.0) + log1p(exp(-fabs(y)));
        double sg = 1.0 / (1.0 + exp(-y));
        double Th = exp(-k * sp), T = exp(-sigma * tau[r]);
        double diff = Th - T;
        loss += diff * diff;
        double dy = 2.0 * diff * (-k * sg * Th) / (double)n;
        double d[64], dn[64];
        grad[M_B4] += dy;
        for (int i = 0; i < 64; ++i) {
            grad[M_W4 + i] += dy * hl[i];
            d[i] = dy * P[M_W4 + i] * silu_grad_d(z[layers - 1][i]);
        }
        for (int l = layers - 1; l >= 0; --l) {
            const int nin = mlp_nin(l);
            const double* W = mlp_w(P, l);
            for (int o = 0; o < 64; ++o) {
                grad[mlp_boff(l) + o] += d[o];
                for (int i = 0; i < nin; ++i) grad[mlp_woff(l) + o * nin + i] += d[o] * h[l][i];
            }
            if (l > 0) {
                for (int i = 0; i < 64; ++i) {
                    double s = 0.0;
                    for (int o = 0; o < 64; ++o) s += W[o * 64 + i] * d[o];
                    dn[i] = s * silu_grad_d(z[l - 1][i]);
                }
                for (int i = 0; i < 64; ++i) d[i] = dn[i];
            }
        }
    }
    return loss / (double)n;
}

/* One Adam step on FP64 state (t = the step number after this update). */
OR_API void or_adam_step(double* w, double* m, double* v, const double* g, int n, double lr,
                         double b1, double b2, double eps, int t) {
    for (int i = 0; i < n; ++i) {
        m[i] = b1 * m[i] + (1.0 - b1) * g[i];
        v[i] = b2 * v[i] + (1.0 - b2) * g[i] * g[i];
        double mh = m[i] / (1.0 - pow(b1, t)), vh = v[i] / (1.0 - pow(b2, t));
        w[i] -= lr * mh / (sqrt(vh) + eps);
    }
}
