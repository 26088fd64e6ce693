// cg_march.cuh -- the view march of the surrogate renderer (texture-filtered
// view samples and fBm) for the persistent renderer's producer warps
// (k_render_mlp_tc).  It emits the samples of k_march's texture-filtered form
// in the same (step, lane) order, so the two renderers' images agree bit for
// bit.
//
// One warp marches one 8x4-pixel region, one ray per lane, the lanes in
// lockstep over the view steps.  A step's inputs -- the occupancy byte of its
// brick, the density/light texel and the fBm texel -- are fetched one step
// ahead of their use, and the two texels of a step together, so that a warp
// waits for one texture latency per step at most instead of the dependent
// chain occupancy -> density -> fBm (the producers are few: each must hide its
// own latency).  The arithmetic (positions, lod, alpha, the transmittance
// update) is k_march's.  k_march keeps its per-step form: with a full grid of
// warps it is faster (0.145 vs 0.174 ms at 1080p, measured).
#pragma once

#include <type_traits>

#include "cg_internal.h"
#include "cg_sample.cuh"

namespace cgm {

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

// One step's inputs: level-0 voxel position v, world position p (for the
// noise), filtered density/light rg and the fBm value nz (valid when rg.x > 0).
struct Step {
    float v0, v1, v2;
    float2 rg;
    float nz;
};

// Fetch step k of the ray (eye + t d, t = tin + (k + 1/2) dt): the same
// positions, lod and sampler calls as the per-step march; the fBm texel is
// fetched beside the density texel whenever the density may be non-zero.
template <bool LOD0>
__device__ __forceinline__ void fetch_step(const VolDesc& vd, const CamDesc& cam,
                                           const TraceParams& tp, float3 d, float tin, float dt,
                                           float vsx, float vsy, float vsz, float pixk,
                                           float t_lod1, int k, bool active, Step& s) {
    s.rg = make_float2(0.f, 0.f);
    s.nz = 0.f;
    s.v0 = s.v1 = s.v2 = 0.f;
    if (!active) return;
    const float t = tin + ((float)k + 0.5f) * dt;
    const float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y, p2 = cam.eye[2] + t * d.z;
    s.v0 = (p0 - vd.wmin[0]) * vsx;
    s.v1 = (p1 - vd.wmin[1]) * vsy;
    s.v2 = (p2 - vd.wmin[2]) * vsz;
    if (LOD0) {
        const float sc = vd.lsc[0];
        const float x = s.v0 * sc, y = s.v1 * sc, z = s.v2 * sc;
        if (cgs::occupied(vd, 0, (int)floorf(x - 0.5f), (int)floorf(y - 0.5f),
                          (int)floorf(z - 0.5f))) {
            s.rg = tex3D<float2>((cudaTextureObject_t)vd.tex[0], x, y, z);
            s.nz = cgs::fbm_volume(tp, p0, p1, p2);
        }
    } else {
        const float lod = t < t_lod1 ? 0.f : log2f(fmaxf(1.f, 2.f * t * pixk));
        s.rg = cgs::quad_hw<true>(vd, s.v0, s.v1, s.v2, lod);
        s.nz = cgs::fbm_volume(tp, p0, p1, p2);
    }
}

// March the region's rays.  For every step at which some lane's sample
// contributes (alpha > 0), on_step(emit, ballot, v0, v1, v2, w, G) is called
// by the whole warp (emit: this lane's sample contributes; w = T * alpha, G =
// the light channel); it returns false to stop the march.  Returns false when
// stopped; T receives the ray's final transmittance.
template <class OnStep>
__device__ __forceinline__ bool march_region(const VolDesc& vd, const CamDesc& cam,
                                             const TraceParams& tp, int px, int py, float& T,
                                             OnStep&& on_step) {
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
    T = 1.f;
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
    bool ok = true;
    // two forms: when every live lane's samples have lod 0 (the warp-uniform
    // common case) level 0 is sampled directly
    auto march = [&](auto lod0_form) {
        constexpr bool LOD0 = decltype(lod0_form)::value;
        Step cur, nxt;
        fetch_step<LOD0>(vd, cam, tp, d, tin, dt, vsx, vsy, vsz, pixk, t_lod1, wkb,
                         live && wkb >= kb && wkb < ke, cur);
        for (int k = wkb; k < Nv; ++k) {
            if (live && k >= ke) live = false;
            if (!__any_sync(0xffffffffu, live)) break;
            // the next step's inputs, in flight while this step is resolved
            fetch_step<LOD0>(vd, cam, tp, d, tin, dt, vsx, vsy, vsz, pixk, t_lod1, k + 1,
                             live && k + 1 >= kb && k + 1 < ke, nxt);
            bool emit = false;
            float w = 0.f, G = 0.f;
            if (live && k >= kb && cur.rg.x > 0.f) {
                const float rho = cur.rg.x * cur.nz;
                if (rho > 0.f) {
                    const float alpha = 1.f - __expf(-tp.sigma * rho * dt);
                    w = T * alpha;
                    G = cur.rg.y;
                    emit = true;
                    T *= 1.f - alpha;
                    if (T < tp.cutoff) live = false;
                }
            }
            const unsigned ballot = __ballot_sync(0xffffffffu, emit);
            if (ballot && !on_step(emit, ballot, cur.v0, cur.v1, cur.v2, w, G)) {
                ok = false;
                return;
            }
            cur = nxt;
        }
    };
    if (__all_sync(0xffffffffu, !live || lod0))
        march(std::true_type{});
    else
        march(std::false_type{});
    return ok;
}

}  // namespace cgm
