// k_deferred.cu -- the deferred renderer: a march pass that records every
// contributing view sample, then shading passes that evaluate the sun term for
// those samples in full warps (exact cone, or the MLP surrogate) and
// accumulate each pixel's colour.
//
// Phase A (k_march): one thread per pixel, one warp per 8x4 pixel tile.  The
// warp marches its rays in lockstep over the view steps; at every step the
// lanes whose sample has alpha > 0 append (voxel position, w = T*alpha,
// light G, lane) to the warp's region of the sample buffer (capacity 32 *
// view_steps), in (step, lane) order.  The pixel's alpha 1 - T is final after
// this pass (one float per pixel; the shading passes write the RGBA image).
// Exact shading (k_shade_exact): one warp per region, 32 samples at a time,
// then each pixel sums its own samples in step order (shuffle broadcast),
// exactly the order of the fused kernel.
// MLP shading: the march also lays the samples out in a flat order (each
// CTA's regions reserve one contiguous range, padded to whole 32-sample
// chunks); a persistent tensor-core kernel (k_shade_mlp_tc) walks that order
// in 128-sample tiles, computing features, running the network and writing
// each sample's contribution to the compact per-slot array; k_accumulate then
// sums each pixel's contributions in step order.
#include <type_traits>

#include "cg_internal.h"
#include "cg_mlp.cuh"
#include "cg_sample.cuh"

namespace {

__device__ __forceinline__ void tile_pixel(int& px, int& py) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    px = blockIdx.x * 16 + (w & 1) * 8 + (lane & 7);
    py = blockIdx.y * 16 + (w >> 1) * 4 + (lane >> 3);
}

// pixel of lane `lane` in region `region` (k_march's mapping)
__device__ __forceinline__ void region_pixel(int region, int lane, int tiles_x, int& px,
                                             int& py) {
    const int blk = region >> 3, w = region & 7;
    px = (blk % tiles_x) * 16 + (w & 1) * 8 + (lane & 7);
    py = (blk / tiles_x) * 16 + (w >> 1) * 4 + (lane >> 3);
}

__device__ __forceinline__ bool pixel_ray(const CamDesc& cam, const VolDesc& vd, int px, int py,
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

// HW: view samples and noise filtered by the texture unit (surrogate renderer).
template <int FMT, bool HW>
__global__ void __launch_bounds__(256) k_march(VolDesc vd, CamDesc cam, TraceParams tp,
                                               SampleBuf sb) {
    // the shading pass may be scheduled once every march CTA has started: its
    // CTAs stage their network while the last wave of the march runs
    grid_dep_trigger();
    int px, py;
    tile_pixel(px, py);
    const int lane = threadIdx.x & 31;
    const int region = (blockIdx.y * gridDim.x + blockIdx.x) * 8 + (threadIdx.x >> 5);
    const bool valid = px < cam.W && py < cam.H;
    float3 d = make_float3(0.f, 0.f, 0.f);
    float tin = 0.f, tout = 0.f;
    bool live = valid && pixel_ray(cam, vd, px, py, d, tin, tout);
    const int Nv = tp.view_steps;
    const float dt = (tout - tin) / (float)Nv;
    const float D = (float)vd.D;
    const float vsx = D / vd.range[0], vsy = D / vd.range[1], vsz = D / vd.range[2];
    const float pixk = cam.tanh / (float)cam.H * vsx;
    // the pixel cone spans less than one voxel before t_lod1: lod is exactly 0
    const float t_lod1 = 0.5f / pixk;
    float T = 1.f;
    unsigned cnt = 0, nsteps = 0;
    float4* pw = sb.pos_w + (size_t)region * sb.capacity;
    float2* gl = sb.light_lane + (size_t)region * sb.capacity;
    // this lane's sampled steps: when every sample has lod 0, steps outside the
    // occupied box read 0 and are skipped (the warp starts at its first one)
    int kb = 0, ke = Nv;
    const bool lod0 = tin + ((float)(Nv - 1) + 0.5f) * dt < t_lod1;
    if (live && lod0) {
        int k0, k1;
        cgs::occupied_steps(vd, cam.eye, d, tin, dt, Nv, k0, k1);
        kb = k0;
        ke = k1 + 1;
        if (kb >= ke) live = false;
    }
    const int wkb = __reduce_min_sync(0xffffffffu, live ? kb : Nv);
    // the steps, in one of two forms: when every live lane's samples have lod
    // 0 (the warp-uniform common case), level 0 is sampled directly (the same
    // texel reads as the lod path at lod 0, without the level arithmetic)
    auto march = [&](auto lod0_form) {
        constexpr bool LOD0 = decltype(lod0_form)::value;
        for (int k = wkb; k < Nv; ++k) {
            if (live && k >= ke) live = false;
            if (!__any_sync(0xffffffffu, live)) break;
            bool emit = false;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f, w = 0.f, G = 0.f;
            if (live && k >= kb) {
                float t = tin + ((float)k + 0.5f) * dt;
                float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y, p2 = cam.eye[2] + t * d.z;
                v0 = (p0 - vd.wmin[0]) * vsx;
                v1 = (p1 - vd.wmin[1]) * vsy;
                v2 = (p2 - vd.wmin[2]) * vsz;
                float2 rg;
                if (LOD0) {
                    rg = cgs::tri_hw<true>(vd, 0, v0, v1, v2);
                } else {
                    float lod = t < t_lod1 ? 0.f : log2f(fmaxf(1.f, 2.f * t * pixk));
                    rg = HW ? cgs::quad_hw<true>(vd, v0, v1, v2, lod)
                            : cgs::quad<FMT, true, true, true>(vd, v0, v1, v2, lod);
                }
                if (rg.x > 0.f) {
                    float rho = rg.x * (HW ? cgs::fbm_volume(tp, p0, p1, p2)
                                           : cgs::fbm(tp, p0, p1, p2));
                    if (rho > 0.f) {
                        float alpha = 1.f - (HW ? __expf(-tp.sigma * rho * dt) : expf(-tp.sigma * rho * dt));
                        w = T * alpha;
                        G = rg.y;
                        emit = true;
                        T *= 1.f - alpha;
                        if (T < tp.cutoff) live = false;
                    }
                }
            }
            const unsigned ballot = __ballot_sync(0xffffffffu, emit);
            if (emit) {
                const unsigned slot = cnt + __popc(ballot & ((1u << lane) - 1u));
                if (CG_IN_BOUNDS((size_t)region * sb.capacity + slot, sb.nslots)) {
                    pw[slot] = make_float4(v0, v1, v2, w);
                    gl[slot] = make_float2(G, __int_as_float(lane));
                }
            }
            // step table: where this step's samples start and which lanes emitted
            if (ballot) {
                if (lane == 0) sb.steps[(size_t)region * Nv + nsteps] = make_uint2(cnt, ballot);
                nsteps++;
            }
            cnt += __popc(ballot);
        }
    };
    if (HW && __all_sync(0xffffffffu, !live || lod0))
        march(std::true_type{});
    else
        march(std::false_type{});
    if (lane == 0) {
        sb.count[region] = cnt;
        sb.nsteps[region] = nsteps;
    }
    if (valid) sb.alpha[(size_t)py * cam.W + px] = 1.f - T;
    // Flat order for the shading pass: the CTA's 8 regions take one contiguous
    // range (reserved with one atomic, padded to whole 32-sample chunks), and
    // every flat row records its sample's slot.
    __shared__ unsigned s_cnt[8], s_base, s_tot;
    const int w = threadIdx.x >> 5;
    if (lane == 0) s_cnt[w] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned tot = 0;
        for (int k = 0; k < 8; ++k) tot += s_cnt[k];
        s_tot = tot;
        s_base = tot ? atomicAdd(sb.flat_total, (tot + 31u) & ~31u) : 0u;
    }
    __syncthreads();
    unsigned o0 = s_base;
    for (int k = 0; k < w; ++k) o0 += s_cnt[k];
    const unsigned slot0 = (unsigned)region * (unsigned)sb.capacity;
    for (unsigned j = lane; j < cnt; j += 32u) sb.slot_of[o0 + j] = slot0 + j;
    if (w == 7) {
        const unsigned end = s_base + s_tot, pad_end = s_base + ((s_tot + 31u) & ~31u);
        if (end + lane < pad_end) sb.slot_of[end + lane] = CG_NO_SLOT;
    }
}

// Sum of each lane's contributions over one chunk of up to 32 samples:
// sample j (held by lane j) belongs to pixel lane lj; pixels accumulate in j
// order with Neumaier compensation.
__device__ __forceinline__ void scatter_chunk(float c, int lj, int m, float& acc, float& comp) {
    const int lane = threadIdx.x & 31;
    for (int j = 0; j < m; ++j) {
        float cj = __shfl_sync(0xffffffffu, c, j);
        int pj = __shfl_sync(0xffffffffu, lj, j);
        if (pj == lane) cgs::neumaier(acc, comp, cj);
    }
}

// The pixel's colour C * sun colour with the alpha the march left in
// `alpha`, stored to `dst` (a device image or the caller's page-locked host
// image).
__device__ __forceinline__ void write_rgb(const float* alpha, float4* dst, const CamDesc& cam,
                                          int px, int py, float C, const TraceParams& tp) {
    if (px < cam.W && py < cam.H) {
        const size_t i = (size_t)py * cam.W + px;
        dst[i] = make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2],
                             alpha[i]);
    }
}

template <int FMT>
__global__ void __launch_bounds__(128) k_shade_exact(VolDesc vd, CamDesc cam, TraceParams tp,
                                                     ConeSchedule cs, SampleBuf sb, int regions,
                                                     int tiles_x, float4* out) {
    const int region = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (region >= regions) return;
    const int lane = threadIdx.x & 31;
    const unsigned n = sb.count[region];
    const float4* pw = sb.pos_w + (size_t)region * sb.capacity;
    const float2* gl = sb.light_lane + (size_t)region * sb.capacity;
    float acc = 0.f, comp = 0.f;
    for (unsigned base = 0; base < n; base += 32) {
        const unsigned i = base + lane;
        float c = 0.f;
        int lj = -1;
        if (i < n) {
            float4 s = pw[i];
            float2 g = gl[i];
            float tau = cgs::sun_cone<FMT>(vd, cs, s.x, s.y, s.z, tp.sun[0], tp.sun[1], tp.sun[2]);
            float L = expf(-tp.sigma * tau) * (tp.ambient + (1.f - tp.ambient) * g.x);
            c = s.w * L;
            lj = __float_as_int(g.y);
        }
        scatter_chunk(c, lj, (int)min(32u, n - base), acc, comp);
    }
    int px, py;
    region_pixel(region, lane, tiles_x, px, py);
    write_rgb(sb.alpha, out, cam, px, py, acc + comp, tp);
}

// Per region: each pixel sums the contributions of its own samples in step
// order, locating them through the march's step table (base slot, ballot).
__global__ void __launch_bounds__(128) k_accumulate(CamDesc cam, TraceParams tp, SampleBuf sb,
                                                    int regions, int tiles_x, int view_steps,
                                                    float4* dst) {
    const int region = blockIdx.x * 4 + (threadIdx.x >> 5);
    grid_dep_wait();  // the contributions of the shading pass
    if (region >= regions) return;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const unsigned ns = sb.nsteps[region];
    const uint2* steps = sb.steps + (size_t)region * view_steps;
    const float* cw = sb.contrib + (size_t)region * sb.capacity;
    float acc = 0.f, comp = 0.f;
    // the step table in coalesced chunks of 32 entries (lane e holds entry e),
    // broadcast by shuffles; eight steps' contributions are fetched before
    // any is summed, and the sums run in step order
    for (unsigned base = 0; base < ns; base += 32u) {
        const unsigned m = min(32u, ns - base);
        const uint2 st_l = lane < (int)m ? steps[base + lane] : make_uint2(0u, 0u);
        for (unsigned e0 = 0; e0 < m; e0 += 8u) {
            float v[8];
            unsigned have = 0u;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int src = (int)(e0 + q) & 31;
                const unsigned sx = __shfl_sync(0xffffffffu, st_l.x, src);
                const unsigned sy = __shfl_sync(0xffffffffu, st_l.y, src);
                v[q] = 0.f;
                // entries past m are (0, 0): no lane emitted there
                if (e0 + q < m && ((sy >> lane) & 1u) &&
                    CG_IN_BOUNDS((size_t)region * sb.capacity + sx + __popc(sy & below),
                                 sb.nslots)) {
                    v[q] = cw[sx + __popc(sy & below)];
                    have |= 1u << q;
                }
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if ((have >> q) & 1u) cgs::neumaier(acc, comp, v[q]);
        }
    }
    int px, py;
    region_pixel(region, lane, tiles_x, px, py);
    write_rgb(sb.alpha, dst, cam, px, py, acc + comp, tp);
}

}  // namespace

static int regions_of(const CamDesc& cam) { return ((cam.W + 15) / 16) * ((cam.H + 15) / 16) * 8; }

cudaError_t launch_march(VolDesc vd, CamDesc cam, TraceParams tp, SampleBuf sb, bool hw,
                         cudaStream_t st) {
    // the flat-order reservation counter starts from zero on every launch
    cudaError_t e = cudaMemsetAsync(sb.flat_total, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    dim3 grd((cam.W + 15) / 16, (cam.H + 15) / 16);
    if (hw)
        k_march<0, true><<<grd, 256, 0, st>>>(vd, cam, tp, sb);
    else if (vd.fmt == 0)
        k_march<0, false><<<grd, 256, 0, st>>>(vd, cam, tp, sb);
    else
        k_march<1, false><<<grd, 256, 0, st>>>(vd, cam, tp, sb);
    return cudaGetLastError();
}

cudaError_t launch_shade_exact(VolDesc vd, CamDesc cam, TraceParams tp, SampleBuf sb,
                               float4* out, cudaStream_t st) {
    ConeSchedule cs = make_cone_schedule(vd, tp);
    const int regions = regions_of(cam), tiles_x = (cam.W + 15) / 16;
    const int blocks = (regions + 3) / 4;
    if (vd.fmt == 0)
        k_shade_exact<0><<<blocks, 128, 0, st>>>(vd, cam, tp, cs, sb, regions, tiles_x, out);
    else
        k_shade_exact<1><<<blocks, 128, 0, st>>>(vd, cam, tp, cs, sb, regions, tiles_x, out);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(CamDesc cam, TraceParams tp, SampleBuf sb, float4* dst,
                              cudaStream_t st) {
    const int regions = regions_of(cam), tiles_x = (cam.W + 15) / 16;
    return launch_dependent(k_accumulate, dim3((regions + 3) / 4), dim3(128), 0, st, cam, tp, sb,
                            regions, tiles_x, (int)tp.view_steps, dst);
}

CG_OOB_TU(k_deferred)
