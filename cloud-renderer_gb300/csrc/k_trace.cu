// k_trace.cu -- per-pixel view march with the exact sun cone (one thread per
// pixel), and the traceCone evaluator.
#include "cg_internal.h"
#include "cg_sample.cuh"

namespace {

// 16x16 pixel tile per 256-thread CTA; each warp owns an 8x4 sub-tile so that
// its rays stay spatially coherent.
__device__ __forceinline__ void tile_pixel(int& px, int& py) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    px = blockIdx.x * 16 + (w & 1) * 8 + (lane & 7);
    py = blockIdx.y * 16 + (w >> 1) * 4 + (lane >> 3);
}

// Ray through the pixel centre and its slab interval against the world box.
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

// Counts (STATS only): [0] view samples evaluated, [1] sun cones, [2] sun-cone
// samples, [3] pixels whose ray met the box.  The counting variant is used
// once, untimed, to derive the algorithmic bytes of a frame.
template <bool STATS>
__device__ __forceinline__ void bump(unsigned long long* stats, int i, unsigned v) {
    if (STATS && v) atomicAdd(stats + i, (unsigned long long)v);
}

template <int FMT, bool STATS>
__global__ void __launch_bounds__(256) k_trace_fused(VolDesc vd, CamDesc cam, TraceParams tp,
                                                     ConeSchedule cs, float4* out,
                                                     unsigned long long* stats) {
    int px, py;
    tile_pixel(px, py);
    if (px >= cam.W || py >= cam.H) return;
    float3 d;
    float tin, tout;
    float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned n_view = 0, n_cone = 0, n_sun = 0, n_hit = 0;
    if (pixel_ray(cam, vd, px, py, d, tin, tout)) {
        n_hit = 1;
        const int Nv = tp.view_steps;
        const float dt = (tout - tin) / (float)Nv;
        const float D = (float)vd.D;
        const float vsx = D / vd.range[0], vsy = D / vd.range[1], vsz = D / vd.range[2];
        const float pixk = cam.tanh / (float)cam.H * vsx;
        // when every sample has lod 0, steps outside the occupied box read 0
        int kbeg = 0, kend = Nv;
        const float tlast = tin + ((float)(Nv - 1) + 0.5f) * dt;
        if (2.f * tlast * pixk <= 1.f) {
            int k0, k1;
            cgs::occupied_steps(vd, cam.eye, d, tin, dt, Nv, k0, k1);
            kbeg = k0;
            kend = k1 + 1;
        }
        float T = 1.f, C = 0.f, Cc = 0.f;
        for (int k = kbeg; k < kend; ++k) {
            float t = tin + ((float)k + 0.5f) * dt;
            float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y, p2 = cam.eye[2] + t * d.z;
            float v0 = (p0 - vd.wmin[0]) * vsx, v1 = (p1 - vd.wmin[1]) * vsy,
                  v2 = (p2 - vd.wmin[2]) * vsz;
            float lod = log2f(fmaxf(1.f, 2.f * t * pixk));
            float2 rg = cgs::quad<FMT, true, true, true>(vd, v0, v1, v2, lod);
            n_view++;
            if (!(rg.x > 0.f)) continue;
            float rho = rg.x * cgs::fbm(tp, p0, p1, p2);
            if (!(rho > 0.f)) continue;
            float alpha = 1.f - expf(-tp.sigma * rho * dt);
            float tau = cgs::sun_cone<FMT>(vd, cs, v0, v1, v2, tp.sun[0], tp.sun[1], tp.sun[2]);
            if (STATS) {
                n_cone++;
                n_sun += cgs::cone_samples(vd, cs, v0, v1, v2, tp.sun[0], tp.sun[1], tp.sun[2]);
            }
            float Ts = expf(-tp.sigma * tau);
            float L = Ts * (tp.ambient + (1.f - tp.ambient) * rg.y);
            cgs::neumaier(C, Cc, T * alpha * L);
            T *= 1.f - alpha;
            if (T < tp.cutoff) break;
        }
        C += Cc;
        res = make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2], 1.f - T);
    }
    out[(size_t)py * cam.W + px] = res;
    bump<STATS>(stats, 0, n_view);
    bump<STATS>(stats, 1, n_cone);
    bump<STATS>(stats, 2, n_sun);
    bump<STATS>(stats, 3, n_hit);
}

// Step i of the reference cone (the light channel, clamp to edge, weight i).
template <int FMT>
__device__ __forceinline__ float quad_split_ref(const VolDesc& vd, const ConeSchedule& cs, int i,
                                                float x, float y, float z) {
    return cgs::quad_split<FMT, true, false, false>(vd, x, y, z, cs.l0[i], cs.frac[i]).y *
           cs.w[i];
}

// One lane's share of a sun cone traced by the whole warp: the weighted
// samples of cone steps lane, lane + 32 (steps that lie beyond the box's
// widened bounds contribute nothing: along the ray they come after the step
// at which the serial cone stops, and none comes back inside).
template <int FMT>
__device__ __forceinline__ float cone_part(const VolDesc& vd, const ConeSchedule& cs, float vx,
                                           float vy, float vz, float sx, float sy, float sz,
                                           int lane) {
    float part = 0.f;
    const float D = (float)vd.D, E = cs.edge;
#pragma unroll
    for (int r = 0; r < CG_MAX_SUN_STEPS / 32; ++r) {
        const int i = lane + 32 * r;
        if (i >= cs.steps) break;
        const float h = cs.h[i];
        const float x = vx + h * sx, y = vy + h * sy, z = vz + h * sz;
        if (cs.mode == 1) {
            part += quad_split_ref<FMT>(vd, cs, i, x, y, z);
        } else if (!(x < -E || y < -E || z < -E || x > D + E || y > D + E || z > D + E)) {
            part += cgs::quad_split<FMT, false, true, true>(vd, x, y, z, cs.l0[i], cs.frac[i]).x *
                    cs.w[i];
        }
    }
    return part;
}

// The fused trace with warp-cooperative sun cones: the warp marches its 32
// rays (an 8x4 tile) in lockstep over the view steps; at a step where at most
// coop_max lanes' samples contribute, the warp traces each of those samples'
// cones in turn, its lanes over the cone steps, the weighted samples summed
// by a shuffle tree; at a step with more, every contributing lane traces its
// own cone as k_trace_fused does.  Samples, opacities and the compositing
// order are k_trace_fused's; only the order in which a cooperative cone's
// terms are added differs.
template <int FMT>
__global__ void __launch_bounds__(256) k_trace_coop(VolDesc vd, CamDesc cam, TraceParams tp,
                                                    ConeSchedule cs, float4* out, int coop_max) {
    int px, py;
    tile_pixel(px, py);
    const int lane = threadIdx.x & 31;
    const bool valid = px < cam.W && py < cam.H;
    float3 d = make_float3(0.f, 0.f, 0.f);
    float tin = 0.f, tout = 0.f;
    const bool hit = valid && pixel_ray(cam, vd, px, py, d, tin, tout);
    bool live = hit;
    const int Nv = tp.view_steps;
    const float dt = (tout - tin) / (float)Nv;
    const float D = (float)vd.D;
    const float vsx = D / vd.range[0], vsy = D / vd.range[1], vsz = D / vd.range[2];
    const float pixk = cam.tanh / (float)cam.H * vsx;
    int kbeg = 0, kend = Nv;
    if (live) {
        const float tlast = tin + ((float)(Nv - 1) + 0.5f) * dt;
        if (2.f * tlast * pixk <= 1.f) {
            int k0, k1;
            cgs::occupied_steps(vd, cam.eye, d, tin, dt, Nv, k0, k1);
            kbeg = k0;
            kend = k1 + 1;
        }
        if (kbeg >= kend) live = false;
    }
    float T = 1.f, C = 0.f, Cc = 0.f;
    const int wk0 = __reduce_min_sync(0xffffffffu, live ? kbeg : Nv);
    for (int k = wk0; k < Nv; ++k) {
        if (live && k >= kend) live = false;
        if (!__any_sync(0xffffffffu, live)) break;
        bool emit = false;
        float v0 = 0.f, v1 = 0.f, v2 = 0.f, alpha = 0.f, G = 0.f;
        if (live && k >= kbeg) {
            const float t = tin + ((float)k + 0.5f) * dt;
            const float p0 = cam.eye[0] + t * d.x, p1 = cam.eye[1] + t * d.y,
                        p2 = cam.eye[2] + t * d.z;
            v0 = (p0 - vd.wmin[0]) * vsx;
            v1 = (p1 - vd.wmin[1]) * vsy;
            v2 = (p2 - vd.wmin[2]) * vsz;
            const float lod = log2f(fmaxf(1.f, 2.f * t * pixk));
            const float2 rg = cgs::quad<FMT, true, true, true>(vd, v0, v1, v2, lod);
            if (rg.x > 0.f) {
                const float rho = rg.x * cgs::fbm(tp, p0, p1, p2);
                if (rho > 0.f) {
                    alpha = 1.f - expf(-tp.sigma * rho * dt);
                    G = rg.y;
                    emit = true;
                }
            }
        }
        const unsigned ballot = __ballot_sync(0xffffffffu, emit);
        if (!ballot) continue;
        float tau = 0.f;
        if (__popc(ballot) <= coop_max) {
            for (unsigned b = ballot; b; b &= b - 1u) {
                const int j = __ffs(b) - 1;
                const float x0 = __shfl_sync(0xffffffffu, v0, j);
                const float x1 = __shfl_sync(0xffffffffu, v1, j);
                const float x2 = __shfl_sync(0xffffffffu, v2, j);
                float part = cone_part<FMT>(vd, cs, x0, x1, x2, tp.sun[0], tp.sun[1], tp.sun[2],
                                            lane);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                if (lane == j) tau = part;
            }
        } else if (emit) {
            tau = cgs::sun_cone<FMT>(vd, cs, v0, v1, v2, tp.sun[0], tp.sun[1], tp.sun[2]);
        }
        if (emit) {
            const float Ts = expf(-tp.sigma * tau);
            const float L = Ts * (tp.ambient + (1.f - tp.ambient) * G);
            cgs::neumaier(C, Cc, T * alpha * L);
            T *= 1.f - alpha;
            if (T < tp.cutoff) live = false;
        }
    }
    C += Cc;
    if (valid)
        out[(size_t)py * cam.W + px] =
            hit ? make_float4(C * tp.sun_color[0], C * tp.sun_color[1], C * tp.sun_color[2],
                              1.f - T)
                : make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int FMT>
__global__ void k_trace_cones(VolDesc vd, TraceParams tp, ConeSchedule cs, const float* pos,
                              int n, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = cgs::sun_cone<FMT>(vd, cs, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], tp.sun[0],
                                tp.sun[1], tp.sun[2]);
}

}  // namespace

// Cone schedule in FP64 on the host (see ConeSchedule).
ConeSchedule make_cone_schedule(const VolDesc& vd, const TraceParams& tp) {
    ConeSchedule cs;
    cs.steps = tp.sun_steps;
    cs.mode = tp.cone_mode;
    cs.edge = (float)vd.D / (float)vd.dims[vd.L - 1];
    const double vw = (double)vd.range[0] / (double)vd.D;
    double h = tp.h0;
    const double maxl = (double)(vd.L - 1);
    for (int i = 0; i < tp.sun_steps && i < CG_MAX_SUN_STEPS; ++i) {
        double r, lod, w;
        if (tp.cone_mode == 1) {
            r = h * (double)tp.tan_half;
            double rr = 2.0 * r > 1.0 ? 2.0 * r : 1.0;
            lod = log2(rr) + (double)tp.lod_offset;
            w = (double)(i + 1) / ((double)tp.sun_steps * (double)tp.down_scaling);
        } else {
            r = h * (double)tp.tan_half;
            if (r < (double)tp.rmin) r = (double)tp.rmin;
            double rr = 2.0 * r > 1.0 ? 2.0 * r : 1.0;
            lod = log2(rr) + (double)tp.lod_offset;
            w = r * vw;
        }
        if (!(lod > 0.0)) lod = 0.0;
        if (lod > maxl) lod = maxl;
        int l0 = (int)floor(lod);
        cs.h[i] = (float)h;
        cs.w[i] = (float)w;
        cs.l0[i] = (unsigned char)l0;
        cs.frac[i] = (float)(lod - (double)l0);
        h += r;
    }
    return cs;
}

cudaError_t launch_trace_fused(VolDesc vd, CamDesc cam, TraceParams tp, float4* out,
                               unsigned long long* stats, cudaStream_t st) {
    ConeSchedule cs = make_cone_schedule(vd, tp);
    dim3 grd((cam.W + 15) / 16, (cam.H + 15) / 16);
    if (!stats && tp.cone_lanes > 0) {
        if (vd.fmt == 0)
            k_trace_coop<0><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, tp.cone_lanes);
        else
            k_trace_coop<1><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, tp.cone_lanes);
    } else if (stats) {
        if (vd.fmt == 0)
            k_trace_fused<0, true><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, stats);
        else
            k_trace_fused<1, true><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, stats);
    } else {
        if (vd.fmt == 0)
            k_trace_fused<0, false><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, nullptr);
        else
            k_trace_fused<1, false><<<grd, 256, 0, st>>>(vd, cam, tp, cs, out, nullptr);
    }
    return cudaGetLastError();
}

namespace {
// Lattice values of every tabulated octave (one thread per entry).
__global__ void k_noise_table(TraceParams tp, float* tab, int total) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int o = 0;
    while (o + 1 < tp.noise_octaves && i >= tp.nt.off[o + 1]) ++o;
    int r = i - tp.nt.off[o];
    const int dx = tp.nt.dim[o][0], dy = tp.nt.dim[o][1];
    int tx = r % dx, ty = (r / dx) % dy, tz = r / (dx * dy);
    tab[i] = cgs::lattice(tp.nt.lo[o][0] + tx, tp.nt.lo[o][1] + ty, tp.nt.lo[o][2] + tz,
                          cgs::octave_key(tp.noise_seed, o));
}
}  // namespace

cudaError_t launch_noise_table(TraceParams tp, float* tab, int total, cudaStream_t st) {
    if (total <= 0) return cudaSuccess;
    k_noise_table<<<(total + 255) / 256, 256, 0, st>>>(tp, tab, total);
    return cudaGetLastError();
}

cudaError_t launch_trace_cones(VolDesc vd, TraceParams tp, const float* pos, int n, float* out,
                               cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    ConeSchedule cs = make_cone_schedule(vd, tp);
    int blocks = (n + 127) / 128;
    if (vd.fmt == 0)
        k_trace_cones<0><<<blocks, 128, 0, st>>>(vd, tp, cs, pos, n, out);
    else
        k_trace_cones<1><<<blocks, 128, 0, st>>>(vd, tp, cs, pos, n, out);
    return cudaGetLastError();
}

CG_OOB_TU(k_trace)
