// k_batch.cu -- many views of many volumes in one persistent launch.
//
// Work unit: one pixel tile of one view.  A view's tiles are numbered after
// the previous views' (tile0 = prefix sum); CTAs take tile numbers from a
// global counter until all are done, and stage the view's descriptors (volume,
// camera, cone schedule) in shared memory when the view changes.
//
// Each tile runs the exact view march of k_trace_fused (same per-sample
// arithmetic in the same order, so images are bit-identical) with one of two
// ray mappings:
//   LPR = 1: one ray per thread (32 rays per warp), 16 x 16 pixels per tile;
//   LPR = 4, 8, 32: LPR lanes per ray (8, 4 or 1 rays per warp): the lanes
//     of a ray evaluate LPR consecutive view steps at once (density, noise,
//     opacity), the group replays the compositing order serially through
//     shuffles to find which steps contribute before the ray terminates, and
//     the contributing steps' sun cones -- the expensive part -- run in
//     parallel across the lanes.
// UNROLL unrolls the step loop (LPR = 1) or the chunk loop (LPR > 1).
#include <algorithm>

#include "cg_internal.h"
#include "cg_sample.cuh"

namespace {

__device__ __forceinline__ bool ray_of(const CamDesc& cam, const VolDesc& vd, int px, int py,
                                       float3& d, float& tin, float& tout) {
    float ndx = (2.f * ((float)px + 0.5f) / (float)cam.W - 1.f) * cam.tanh * cam.aspect;
    float ndy = (1.f - 2.f * ((float)py + 0.5f) / (float)cam.H) * cam.tanh;
    float dx = cam.f[0] + ndx * cam.s[0] + ndy * cam.u[0];
    float dy = cam.f[1] + ndx * cam.s[1] + ndy * cam.u[1];
    float dz = cam.f[2] + ndx * cam.s[2] + ndy * cam.u[2];
    float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
    d = make_float3(dx * inv, dy * inv, dz * inv);
    float dd[3] = {d.x, d.y, d.z};
    float tmin = -1e30f, tmax = 1e30f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float lo = vd.wmin[a], hi = vd.wmin[a] + vd.range[a];
        if (dd[a] == 0.f) {
            if (cam.eye[a] < lo || cam.eye[a] > hi) return false;
            continue;
        }
        float iv = 1.f / dd[a];
        float t0 = (lo - cam.eye[a]) * iv, t1 = (hi - cam.eye[a]) * iv;
        tmin = fmaxf(tmin, fminf(t0, t1));
        tmax = fminf(tmax, fmaxf(t0, t1));
    }
    tin = fmaxf(tmin, 0.f);
    tout = tmax;
    return tout > tin;
}

// Pixel tile of a CTA: 256 / LPR pixels, 16 wide for LPR = 1 (16 x 16),
// otherwise 8 wide (8 x 32 / LPR).
template <int LPR>
struct TileShape {
    static constexpr int W = LPR == 1 ? 16 : 8;
    static constexpr int H = (256 / LPR) / W;
};

// The march of one ray, one thread (k_trace_fused's loop).
template <int FMT, int UNROLL>
__device__ __forceinline__ float4 march_thread(const VolDesc& vd, const CamDesc& cam,
                                               const TraceParams& tp, const ConeSchedule& cs,
                                               int px, int py) {
    float3 d;
    float tin, tout;
    if (!ray_of(cam, vd, px, py, d, tin, tout)) return make_float4(0.f, 0.f, 0.f, 0.f);
    const int Nv = tp.view_steps;
    const float dt = (tout - tin) / (float)Nv;
    const float D = (float)vd.D;
    const float vsx = D / vd.range[0], vsy = D / vd.range[1], vsz = D / vd.range[2];
    const float pixk = cam.tanh / (float)cam.H * vsx;
    // when every sample has lod 0, steps outside the occupied box read 0
    int kbeg = 0, kend = Nv;
    if (2.f * (tin + ((float)(Nv - 1) + 0.5f) * dt) * pixk <= 1.f) {
        int k0, k1;
        cgs::occupied_steps(vd, cam.eye, d, tin, dt, Nv, k0, k1);
        kbeg = k0;
        kend = k1 + 1;
    }
    float T = 1.f, C = 0.f, Cc = 0.f;
#pragma unroll UNROLL
    for (int k = kbeg; k < kend; ++k) {
        float t = tin + ((float)k + 0.5f) * dt;
        float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y, p2 = cam.eye[2] + t * d.z;
        float v0 = (p0 - vd.wmin[0]) * vsx, v1 = (p1 - vd.wmin[1]) * vsy,
              v2 = (p2 - vd.wmin[2]) * vsz;
        float lod = log2f(fmaxf(1.f, 2.f * t * pixk));
        float2 rg = cgs::quad<FMT, true, true, true>(vd, v0, v1, v2, lod);
        if (!(rg.x > 0.f)) continue;
        float rho = rg.x * cgs::fbm(tp, p0, p1, p2);
        if (!(rho > 0.f)) continue;
        float alpha = 1.f - expf(-tp.sigma * rho * dt);
        float tau = cgs::sun_cone<FMT>(vd, cs, v0, v1, v2, tp.sun[0], tp.sun[1], tp.sun[2]);
        float Ts = expf(-tp.sigma * tau);
        float L = Ts * (tp.ambient + (1.f - tp.ambient) * rg.y);
        cgs::neumaier(C, Cc, T * alpha * L);
        T *= 1.f - alpha;
        if (T < tp.cutoff) break;
    }
    C += Cc;
    return make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2], 1.f - T);
}

// The march of one ray by LPR lanes (see the file comment).  All lanes of the
// warp call it together; `live` marks lanes of a group with a real pixel.
template <int FMT, int LPR, int UNROLL>
__device__ __forceinline__ float4 march_group(const VolDesc& vd, const CamDesc& cam,
                                              const TraceParams& tp, const ConeSchedule& cs,
                                              int px, int py, bool pixel_ok) {
    const int lane = threadIdx.x & 31, j = lane & (LPR - 1), g0 = lane - j;
    float3 d = make_float3(0.f, 0.f, 0.f);
    float tin = 0.f, tout = 0.f;
    bool hit = pixel_ok && ray_of(cam, vd, px, py, d, tin, tout);
    const int Nv = tp.view_steps;
    const float dt = (tout - tin) / (float)Nv;
    const float D = (float)vd.D;
    const float vsx = D / vd.range[0], vsy = D / vd.range[1], vsz = D / vd.range[2];
    const float pixk = cam.tanh / (float)cam.H * vsx;
    // when every sample has lod 0, steps outside the occupied box read 0: the
    // group starts at the box's first step (rounded down to whole groups of
    // steps) and ends after its last
    int kbeg = 0, kend = Nv;
    if (hit && 2.f * (tin + ((float)(Nv - 1) + 0.5f) * dt) * pixk <= 1.f) {
        int k0, k1;
        cgs::occupied_steps(vd, cam.eye, d, tin, dt, Nv, k0, k1);
        kbeg = k0;
        kend = k1 + 1;
    }
    float T = 1.f, C = 0.f, Cc = 0.f;
    bool run = hit && kbeg < kend;  // the group's ray has not terminated
    const int base0 = __reduce_min_sync(0xffffffffu, run ? kbeg - kbeg % LPR : Nv);
#pragma unroll UNROLL
    for (int base = base0; base < Nv; base += LPR) {
        if (!__any_sync(0xffffffffu, run)) break;
        // ---- this lane's step: position, density, noise, opacity
        const int k = base + j;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f, alpha = 0.f, G = 0.f;
        if (run && k < kend) {
            float t = tin + ((float)k + 0.5f) * dt;
            float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y, p2 = cam.eye[2] + t * d.z;
            v0 = (p0 - vd.wmin[0]) * vsx;
            v1 = (p1 - vd.wmin[1]) * vsy;
            v2 = (p2 - vd.wmin[2]) * vsz;
            float lod = log2f(fmaxf(1.f, 2.f * t * pixk));
            float2 rg = cgs::quad<FMT, true, true, true>(vd, v0, v1, v2, lod);
            if (rg.x > 0.f) {
                float rho = rg.x * cgs::fbm(tp, p0, p1, p2);
                if (rho > 0.f) {
                    alpha = 1.f - expf(-tp.sigma * rho * dt);
                    G = rg.y;
                }
            }
        }
        // ---- compositing order, replayed by every lane of the group: the
        // transmittance in front of this lane's step, and whether the ray is
        // still running there
        float Tfront = T, Tg = T;
        bool mine = false, going = run;
#pragma unroll
        for (int i = 0; i < LPR; ++i) {
            const float ai = __shfl_sync(0xffffffffu, alpha, g0 + i);
            const bool contributes = going && ai > 0.f;
            if (i == j) {
                Tfront = Tg;
                mine = contributes;
            }
            if (contributes) {
                Tg *= 1.f - ai;
                if (Tg < tp.cutoff) going = false;
            }
        }
        // ---- the contributing steps' sun cones, in parallel
        float term = 0.f;
        if (mine) {
            float tau = cgs::sun_cone<FMT>(vd, cs, v0, v1, v2, tp.sun[0], tp.sun[1], tp.sun[2]);
            float Ts = expf(-tp.sigma * tau);
            float L = Ts * (tp.ambient + (1.f - tp.ambient) * G);
            term = Tfront * alpha * L;
        }
        // ---- accumulate in step order
#pragma unroll
        for (int i = 0; i < LPR; ++i) {
            const float ti = __shfl_sync(0xffffffffu, term, g0 + i);
            const bool ci = __shfl_sync(0xffffffffu, mine, g0 + i);
            if (ci) cgs::neumaier(C, Cc, ti);
        }
        T = Tg;
        run = going && base + LPR < kend;
    }
    C += Cc;
    if (!hit) return make_float4(0.f, 0.f, 0.f, 0.f);
    return make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2], 1.f - T);
}

template <int FMT, int LPR, int UNROLL>
__global__ void __launch_bounds__(256) k_trace_batch(const BatchView* views, int nviews,
                                                     unsigned total_tiles, unsigned* counter) {
    __shared__ BatchView sv;
    __shared__ unsigned s_tile;
    __shared__ int s_view;
    using TS = TileShape<LPR>;
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned t = atomicAdd(counter, 1u);
            int v = -1;
            if (t < total_tiles) {
                // last view whose first tile is <= t
                int lo = 0, hi = nviews - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (views[mid].tile0 <= t) lo = mid;
                    else hi = mid - 1;
                }
                v = lo;
            }
            s_tile = t;
            s_view = v;
        }
        __syncthreads();
        const int v = s_view;
        const unsigned t = s_tile;
        if (v < 0) break;
        if (v != cur) {
            // stage the view's descriptors (words, all threads)
            const uint32_t* src = reinterpret_cast<const uint32_t*>(views + v);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&sv);
            for (int i = threadIdx.x; i < (int)(sizeof(BatchView) / 4); i += blockDim.x)
                dst[i] = src[i];
            cur = v;
        }
        __syncthreads();
        const unsigned local = t - sv.tile0;
        const int tx = (int)(local % (unsigned)sv.tiles_x), ty = (int)(local / (unsigned)sv.tiles_x);
        if (LPR == 1) {
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            const int px = tx * 16 + (w & 1) * 8 + (lane & 7);
            const int py = ty * 16 + (w >> 1) * 4 + (lane >> 3);
            if (px < sv.cam.W && py < sv.cam.H)
                sv.out[(size_t)py * sv.cam.W + px] =
                    march_thread<FMT, UNROLL>(sv.vd, sv.cam, sv.tp, sv.cs, px, py);
        } else {
            const int r = threadIdx.x / LPR;  // ray of the tile
            const int px = tx * TS::W + r % TS::W, py = ty * TS::H + r / TS::W;
            const bool ok = px < sv.cam.W && py < sv.cam.H;
            const float4 res = march_group<FMT, LPR, UNROLL>(sv.vd, sv.cam, sv.tp, sv.cs, px, py, ok);
            if (ok && (threadIdx.x & (LPR - 1)) == 0) sv.out[(size_t)py * sv.cam.W + px] = res;
        }
        __syncthreads();  // sv / s_tile are rewritten by the next iteration
    }
}

template <int FMT, int LPR, int UNROLL>
cudaError_t launch_one(const BatchView* views, int n, unsigned total, unsigned* counter,
                       int blocks, cudaStream_t st) {
    k_trace_batch<FMT, LPR, UNROLL><<<blocks, 256, 0, st>>>(views, n, total, counter);
    return cudaGetLastError();
}

template <int FMT, int LPR>
cudaError_t launch_unroll(int unroll, const BatchView* views, int n, unsigned total,
                          unsigned* counter, int blocks, cudaStream_t st) {
    switch (unroll) {
        case 2: return launch_one<FMT, LPR, 2>(views, n, total, counter, blocks, st);
        case 4: return launch_one<FMT, LPR, 4>(views, n, total, counter, blocks, st);
        default: return launch_one<FMT, LPR, 1>(views, n, total, counter, blocks, st);
    }
}

template <int FMT>
cudaError_t launch_lpr(int lpr, int unroll, const BatchView* views, int n, unsigned total,
                       unsigned* counter, int blocks, cudaStream_t st) {
    switch (lpr) {
        case 4: return launch_unroll<FMT, 4>(unroll, views, n, total, counter, blocks, st);
        case 8: return launch_unroll<FMT, 8>(unroll, views, n, total, counter, blocks, st);
        case 32: return launch_unroll<FMT, 32>(unroll, views, n, total, counter, blocks, st);
        default: return launch_unroll<FMT, 1>(unroll, views, n, total, counter, blocks, st);
    }
}

}  // namespace

void batch_tiles(int lanes_per_ray, int width, int height, int& tiles_x, int& tiles_y) {
    const int tw = lanes_per_ray == 1 ? 16 : 8;
    const int th = (256 / lanes_per_ray) / tw;
    tiles_x = (width + tw - 1) / tw;
    tiles_y = (height + th - 1) / th;
}

cudaError_t launch_trace_batch(int fmt, int lanes_per_ray, int unroll, const BatchView* views,
                               int n, unsigned total_tiles, unsigned* counter, cudaStream_t st) {
    if (n <= 0 || total_tiles == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    // persistent: a few CTAs per SM pull tiles until the counter runs out
    const int blocks = (int)std::min<unsigned>(total_tiles, (unsigned)sms * 8u);
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    return fmt == 0 ? launch_lpr<0>(lanes_per_ray, unroll, views, n, total_tiles, counter, blocks, st)
                    : launch_lpr<1>(lanes_per_ray, unroll, views, n, total_tiles, counter, blocks, st);
}

CG_OOB_TU(k_batch)
